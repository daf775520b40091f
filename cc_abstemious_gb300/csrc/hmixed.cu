// Mixed form over H-matrix operators (the Hierarchical solver of solve.rs:74-150
// with FP32 storage): every frequency's operator is compressed by the ACA
// build of hmatrix.cu (FP64 adaptive cross approximation with the reference's
// pivot stream, then QR + SVD recompression, aca.rs:57-179), and its leaves
// are repacked here as complex FP32 in cluster order:
//
//   * the unknowns are permuted so that every cluster of the tree is one
//     contiguous index range (the leaves in depth-first order), so a block's
//     rows and columns are ranges and its operand slices are contiguous;
//   * dense leaves: m x n column-major; admissible leaves: U (m x r) then V
//     (n x r), column-major, r the recompressed rank (A_b ~ U V^T, aca.rs:
//     181-195 applies it as U (V^T x)).
//
// The batched mat-vec W_s = A_s v_s (h_matrix.rs:218-234) of every active
// system runs in four launches:
//   gather   v_s in cluster order, split into FP32 hi + lo parts;
//   project  t_b = V_b^T v[cols_b], one warp per group of four rank columns
//            of every admissible block (a flat list per operator);
//   rows     for every leaf row cluster (<= 64 rows), the blocks that cover it
//            in chunks of eight, one warp per block: its dense rows times
//            v[cols] or its U rows times t_b, the chunk's sum stored apart;
//   reduce   every cluster's chunk sums added in chunk order and written back
//            in the original order (no atomics, a fixed order).
// Each stored FP32 entry is read once per mat-vec: the kernel is bound by HBM
// bandwidth (8 B per stored entry).  Products are FP32; Krylov mat-vecs fold
// partial sums of 16 terms into FP64, residual mat-vecs (START / CHECK) split
// every product exactly and accumulate in float-float, as the dense mixed
// form does.  Systems sharing an operator (several incident waves) read it
// separately.
//
// Block-Jacobi preconditioning uses the dense diagonal leaves: their FP32
// inverses (Gauss-Jordan with partial pivoting) applied per cluster.
#include <algorithm>
#include <cmath>
#include <memory>

#include "common.cuh"
#include "complex.cuh"
#include "gmres.cuh"
#include "hmatrix.cuh"
#include "tree.cuh"
#include "hmixed.cuh"

namespace bem {

namespace {

struct HmBlock {
    int64_t r0, m, c0, n;  // permuted row / column ranges
    int32_t adm, pad;
};

struct HmDev {
    int nb, nadm, nrc, R;
    int64_t n, ttot;
    const HmBlock* blk;
    const int32_t* adm_list;
    const int64_t* off;    // [op * nb + b] store offset (complex entries)
    const int32_t* rank;   // [op * nb + b]
    const int64_t* toff;   // [op * nb + b] offset of t_b within a system's projections
    const float2* store;
    const int64_t* rc_start;  // nrc + 1 cluster bounds (permuted)
    const int32_t* rc_ptr;    // nrc + 1 into the item lists
    const int32_t* item_blk;
    const int32_t* item_row;  // the cluster's first row, local to the block
    const int64_t* perm;      // permuted position -> original index
    float2 *xh, *xl;          // nsys x n gathered operand, hi + lo
    float4* t;                // nsys x ttot projections, float-float (re hi, im hi, re lo, im lo)
    const struct HmItem* items;  // [op * nitems + it]: the rows pass, packed
    int64_t nitems;
    const struct HmProj* proj;   // [op * pstride + q]: one per rank column
    int64_t pstride;
    const int32_t* nproj;        // [op]: rank columns of the operator
    const int32_t* ch_rc;        // [chunk]: cluster of a chunk of items
    const int32_t* ch_it;        // [chunk + 1]: the chunk's items
    const int32_t* rc_ch;        // [cluster + 1]: the cluster's chunks
    int64_t nchunks;
    float4* part;                // nsys x nchunks x 64 partial row sums (float-float)
};

// One block's contribution to one row cluster, packed for a single load: the
// block's data at `off` (dense: m x n; low-rank: U, m x r), its leading
// dimension m, len = n (dense) or r (low-rank), the cluster's first row local
// to the block, and the operand: columns from c0 (dense) or the projections
// from toff (low-rank).
struct HmItem {
    int64_t off, src;  // store offset; c0 (dense) or toff (low-rank)
    int32_t ld, len, lr, adm;
};

// Up to PJ_COLS consecutive rank columns k .. k + cnt of one admissible
// block: V's column k at voff (columns n entries apart), the block's first
// column c0, and the projection slot of column k.
constexpr int PJ_COLS = 4;
struct HmProj {
    int64_t voff, c0, t;
    int32_t n, cnt;
};

__device__ __forceinline__ void two_sum_f(float a, float b, float& s, float& e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// (hi, lo) += a * b: the product split exactly by an FMA, summed in float-float.
__device__ __forceinline__ void ff_acc2(float& hi, float& lo, float a, float b) {
    const float p = a * b;
    const float e = fmaf(a, b, -p);
    float s, err;
    two_sum_f(hi, p, s, err);
    hi = s;
    lo += err + e;
}

// Accumulator of a complex sum of FP32 products with an operand split into
// hi + lo floats, in FP32 arithmetic only (GB300 runs FP64 at ~1/64 of the
// FP32 rate, so FP64 in these streaming loops would bound them): EXACT --
// every product split exactly by an FMA, float-float sums (residuals);
// otherwise FP32 sums of FOLD terms folded into float-float (Krylov vectors).
constexpr int FOLD = 16;

// (h, l) += (h2, l2), renormalised.
__device__ __forceinline__ void ff_add(float& h, float& l, float h2, float l2) {
    float s, e;
    two_sum_f(h, h2, s, e);
    e += l + l2;
    h = s + e;
    l = e - (h - s);
}

template <int EXACT>
struct CAcc {
    float rh = 0, rl = 0, ih = 0, il = 0;  // float-float real and imaginary sums
    float pr = 0, pi = 0;                  // FAST: the open FP32 partial sums
    int cnt = 0;
    __device__ __forceinline__ void add(float2 a, float2 xh, float2 xl) {
        if (EXACT) {
            ff_acc2(rh, rl, a.x, xh.x);
            ff_acc2(rh, rl, -a.y, xh.y);
            ff_acc2(ih, il, a.x, xh.y);
            ff_acc2(ih, il, a.y, xh.x);
            rl = fmaf(a.x, xl.x, fmaf(-a.y, xl.y, rl));
            il = fmaf(a.x, xl.y, fmaf(a.y, xl.x, il));
        } else {
            pr = fmaf(a.x, xh.x, fmaf(-a.y, xh.y, pr));
            pi = fmaf(a.x, xh.y, fmaf(a.y, xh.x, pi));
            if (++cnt == FOLD) fold();
        }
    }
    __device__ __forceinline__ void fold() {
        float s, e;
        two_sum_f(rh, pr, s, e);
        rh = s;
        rl += e;
        two_sum_f(ih, pi, s, e);
        ih = s;
        il += e;
        pr = pi = 0.f;
        cnt = 0;
    }
    // the sum as float-float: (re hi, im hi, re lo, im lo)
    __device__ __forceinline__ float4 ff() {
        if (!EXACT) fold();
        return make_float4(rh, ih, rl, il);
    }
};

// Sum of a float-float complex value over the 32 lanes of a warp.
__device__ __forceinline__ float4 warp_ff_sum(float4 v) {
    for (int o = 16; o > 0; o >>= 1) {
        const float hx = __shfl_xor_sync(0xffffffffu, v.x, o), hy = __shfl_xor_sync(0xffffffffu, v.y, o);
        const float lx = __shfl_xor_sync(0xffffffffu, v.z, o), ly = __shfl_xor_sync(0xffffffffu, v.w, o);
        ff_add(v.x, v.z, hx, lx);
        ff_add(v.y, v.w, hy, ly);
    }
    return v;
}

__device__ __forceinline__ double2 ff_to_double(float4 v) {
    return make_double2((double)v.x + (double)v.z, (double)v.y + (double)v.w);
}

__device__ __forceinline__ const double2* hm_operand(const GmBatch& bt, const GmState& st, int s, int mode) {
    const GmView g = gm_view(bt, s);
    const double2* kv = bt.Z ? bt.Z : bt.Q;
    return mode == MV_Q ? kv + g.q + (size_t)st.k * g.n : bt.X + g.v;
}

__global__ void hmx_gather_kernel(HmDev h, GmBatch bt, int mode) {
    const int s = blockIdx.y;
    const GmState& st = bt.st[s];
    if (!gm_apply_active(bt, st, mode)) return;
    const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= h.n) return;
    const double2 x = hm_operand(bt, st, s, mode)[h.perm[q]];
    const float hx = (float)x.x, hy = (float)x.y;
    h.xh[(size_t)s * h.n + q] = make_float2(hx, hy);
    h.xl[(size_t)s * h.n + q] = make_float2((float)(x.x - (double)hx), (float)(x.y - (double)hy));
}

constexpr int PJ_WARPS = 8;

// t_b[k] = V_b[:, k]^T v[cols_b]: one warp per group of up to PJ_COLS rank
// columns of an admissible block (a flat list per operator), lanes along
// the columns, the group's loads in flight together.
template <int EXACT>
__global__ void __launch_bounds__(PJ_WARPS * 32) hmx_project_kernel(HmDev h, GmBatch bt, int mode) {
    const int s = blockIdx.y;
    if (!gm_apply_active(bt, bt.st[s], mode)) return;
    const int op = s / h.R;
    const int64_t q = (int64_t)blockIdx.x * PJ_WARPS + (threadIdx.x >> 5);
    if (q >= h.nproj[op]) return;
    const int lane = threadIdx.x & 31;
    const HmProj P = h.proj[(size_t)op * h.pstride + q];
    const float2* v0 = h.store + P.voff;
    const float2* xh = h.xh + (size_t)s * h.n + P.c0;
    const float2* xl = h.xl + (size_t)s * h.n + P.c0;
    CAcc<EXACT> acc[PJ_COLS];
    for (int64_t j = lane; j < P.n; j += 32) {
        float2 a[PJ_COLS];
#pragma unroll
        for (int c = 0; c < PJ_COLS; ++c)
            a[c] = c < P.cnt ? __ldcs(v0 + (size_t)c * P.n + j) : make_float2(0.f, 0.f);
        const float2 x1 = xh[j], x2 = xl[j];
#pragma unroll
        for (int c = 0; c < PJ_COLS; ++c)
            if (c < P.cnt) acc[c].add(a[c], x1, x2);
    }
#pragma unroll
    for (int c = 0; c < PJ_COLS; ++c) {
        if (c >= P.cnt) break;  // uniform over the warp
        const float4 v = warp_ff_sum(acc[c].ff());
        if (lane == 0) h.t[(size_t)s * h.ttot + P.t + c] = v;
    }
}

constexpr int RW_ROWS = 64, RW_WARPS = 8, RW_THREADS = RW_WARPS * 32;

// Partial row sums of one chunk of a cluster's items (up to RW_WARPS): one
// warp per item, each lane two rows (lane, lane + 32); the warps' sums are
// added in shared memory and stored as the chunk's partial.  Clusters hold
// at most RW_ROWS rows (leaf size <= 64, checked on the host).
template <int EXACT>
__global__ void __launch_bounds__(RW_THREADS) hmx_rows_kernel(HmDev h, GmBatch bt, int mode) {
    const int s = blockIdx.y;
    if (!gm_apply_active(bt, bt.st[s], mode)) return;
    __shared__ float4 red[RW_WARPS][RW_ROWS];
    const int64_t ch = blockIdx.x;
    const int rc = h.ch_rc[ch], op = s / h.R;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int rows = (int)(h.rc_start[rc + 1] - h.rc_start[rc]);
    const bool oka = lane < rows, okb = lane + 32 < rows;
    CAcc<EXACT> acc_a, acc_b;
    const int it = h.ch_it[ch] + warp;
    if (it < h.ch_it[ch + 1]) {
        const HmItem I = h.items[(size_t)op * h.nitems + it];
        const float2* D = h.store + I.off + I.lr;
        if (!I.adm) {
            const float2* xa = h.xh + (size_t)s * h.n + I.src;
            const float2* xb = h.xl + (size_t)s * h.n + I.src;
            int j = 0;
            for (; j + 4 <= I.len; j += 4) {
                float2 a[4], b[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    a[u] = oka ? __ldcs(D + (size_t)(j + u) * I.ld + lane) : make_float2(0.f, 0.f);
                    b[u] = okb ? __ldcs(D + (size_t)(j + u) * I.ld + lane + 32) : make_float2(0.f, 0.f);
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const float2 x1 = xa[j + u], x2 = xb[j + u];
                    acc_a.add(a[u], x1, x2);
                    acc_b.add(b[u], x1, x2);
                }
            }
            for (; j < I.len; ++j) {
                const float2 a = oka ? __ldcs(D + (size_t)j * I.ld + lane) : make_float2(0.f, 0.f);
                const float2 b = okb ? __ldcs(D + (size_t)j * I.ld + lane + 32) : make_float2(0.f, 0.f);
                acc_a.add(a, xa[j], xb[j]);
                acc_b.add(b, xa[j], xb[j]);
            }
        } else {
            const float4* t = h.t + (size_t)s * h.ttot + I.src;
            int k = 0;
            for (; k + 4 <= I.len; k += 4) {
                float2 a[4], b[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    a[u] = oka ? __ldcs(D + (size_t)(k + u) * I.ld + lane) : make_float2(0.f, 0.f);
                    b[u] = okb ? __ldcs(D + (size_t)(k + u) * I.ld + lane + 32) : make_float2(0.f, 0.f);
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const float4 tk = t[k + u];
                    const float2 th = make_float2(tk.x, tk.y), tl = make_float2(tk.z, tk.w);
                    acc_a.add(a[u], th, tl);
                    acc_b.add(b[u], th, tl);
                }
            }
            for (; k < I.len; ++k) {
                const float4 tk = t[k];
                const float2 th = make_float2(tk.x, tk.y), tl = make_float2(tk.z, tk.w);
                const float2 a = oka ? __ldcs(D + (size_t)k * I.ld + lane) : make_float2(0.f, 0.f);
                const float2 b = okb ? __ldcs(D + (size_t)k * I.ld + lane + 32) : make_float2(0.f, 0.f);
                acc_a.add(a, th, tl);
                acc_b.add(b, th, tl);
            }
        }
    }
    red[warp][lane] = acc_a.ff();
    red[warp][lane + 32] = acc_b.ff();
    __syncthreads();
    if (threadIdx.x < RW_ROWS) {
        float4 v = red[0][threadIdx.x];
        for (int w = 1; w < RW_WARPS; ++w) {
            const float4 u = red[w][threadIdx.x];
            ff_add(v.x, v.z, u.x, u.z);
            ff_add(v.y, v.w, u.y, u.w);
        }
        h.part[((size_t)s * h.nchunks + ch) * RW_ROWS + threadIdx.x] = v;
    }
}

// W[rows of cluster rc] = the cluster's chunk partials, added in chunk order.
__global__ void __launch_bounds__(RW_ROWS) hmx_reduce_kernel(HmDev h, GmBatch bt, int mode) {
    const int s = blockIdx.y;
    if (!gm_apply_active(bt, bt.st[s], mode)) return;
    const int rc = blockIdx.x, i = threadIdx.x;
    const int64_t rs = h.rc_start[rc];
    if (i >= (int)(h.rc_start[rc + 1] - rs)) return;
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int ch = h.rc_ch[rc]; ch < h.rc_ch[rc + 1]; ++ch) {
        const float4 p = h.part[((size_t)s * h.nchunks + ch) * RW_ROWS + i];
        ff_add(v.x, v.z, p.x, p.z);
        ff_add(v.y, v.w, p.y, p.w);
    }
    const GmView g = gm_view(bt, s);
    bt.W[g.v + h.perm[rs + i]] = ff_to_double(v);
}

// Repacking of one FP64 leaf into FP32 cluster order (one CTA per leaf).
struct RepackLeaf {
    int64_t row_off, col_off, src, dst, m, n, r0, c0;
    int32_t adm, rank;
};

__global__ void hmx_repack_kernel(const RepackLeaf* __restrict__ L, const int64_t* __restrict__ rows,
                                  const int64_t* __restrict__ cols, const int64_t* __restrict__ pos,
                                  const double2* __restrict__ src, float2* __restrict__ dst) {
    const RepackLeaf l = L[blockIdx.x];
    const double2* S = src + l.src;
    float2* D = dst + l.dst;
    if (!l.adm) {
        for (int64_t e = threadIdx.x; e < l.m * l.n; e += blockDim.x) {
            const int64_t i = e % l.m, j = e / l.m;
            const int64_t ip = pos[rows[l.row_off + i]] - l.r0, jp = pos[cols[l.col_off + j]] - l.c0;
            const double2 v = S[j * l.m + i];
            D[jp * l.m + ip] = make_float2((float)v.x, (float)v.y);
        }
    } else {
        // U: m x kmax in the source (first rank columns used), m x rank here;
        // V follows in hmx_repack_v_kernel
        for (int64_t e = threadIdx.x; e < l.m * l.rank; e += blockDim.x) {
            const int64_t i = e % l.m, k = e / l.m;
            const double2 v = S[k * l.m + i];
            D[k * l.m + (pos[rows[l.row_off + i]] - l.r0)] = make_float2((float)v.x, (float)v.y);
        }
    }
}

__global__ void hmx_repack_v_kernel(const RepackLeaf* __restrict__ L, const int32_t* __restrict__ kmaxs,
                                    const int64_t* __restrict__ cols, const int64_t* __restrict__ pos,
                                    const double2* __restrict__ src, float2* __restrict__ dst) {
    const RepackLeaf l = L[blockIdx.x];
    if (!l.adm) return;
    const double2* S = src + l.src + (size_t)l.m * kmaxs[blockIdx.x];
    float2* D = dst + l.dst + (size_t)l.m * l.rank;
    for (int64_t e = threadIdx.x; e < l.n * l.rank; e += blockDim.x) {
        const int64_t j = e % l.n, k = e / l.n;
        const double2 v = S[k * l.n + j];
        D[k * l.n + (pos[cols[l.col_off + j]] - l.c0)] = make_float2((float)v.x, (float)v.y);
    }
}

// ---------------------------------------------------------------------------
// Block-Jacobi on the diagonal leaves: [D | I] reduced by Gauss-Jordan with
// partial pivoting (FP32), one CTA per (cluster, operator).
constexpr int BJ_MAX = 64;

constexpr int BJ_STRIDE = 2 * BJ_MAX + 1;
constexpr size_t BJ_SMEM = sizeof(float2) * BJ_MAX * BJ_STRIDE;

__global__ void __launch_bounds__(256) hmx_bj_invert_kernel(HmDev h, const int32_t* __restrict__ diag_blk,
                                                            float2* __restrict__ Minv, int* __restrict__ small) {
    extern __shared__ float2 aug_raw[];  // BJ_MAX rows of BJ_STRIDE
    auto aug = reinterpret_cast<float2(*)[BJ_STRIDE]>(aug_raw);
    __shared__ int piv;
    const int rc = blockIdx.x, op = blockIdx.y;
    const int b = (int)(h.rc_start[rc + 1] - h.rc_start[rc]);
    const int db = diag_blk[rc];
    const float2* D = h.store + h.off[(size_t)op * h.nb + db];
    for (int e = threadIdx.x; e < b * 2 * b; e += blockDim.x) {
        const int i = e / (2 * b), j = e % (2 * b);
        aug[i][j] = j < b ? D[(size_t)j * b + i] : make_float2(j - b == i ? 1.f : 0.f, 0.f);
    }
    __syncthreads();
    for (int c = 0; c < b; ++c) {
        if (threadIdx.x == 0) {
            int best = c;
            float bv = -1.f;
            for (int r = c; r < b; ++r) {
                const float v = fabsf(aug[r][c].x) + fabsf(aug[r][c].y);
                if (v > bv) { bv = v; best = r; }
            }
            piv = best;
            if (!(bv > 0.f)) atomicAdd(small, 1);
        }
        __syncthreads();
        const int p = piv;
        if (p != c)
            for (int j = threadIdx.x; j < 2 * b; j += blockDim.x) {
                const float2 tmp = aug[c][j];
                aug[c][j] = aug[p][j];
                aug[p][j] = tmp;
            }
        __syncthreads();
        float2 d = aug[c][c];
        float dn = d.x * d.x + d.y * d.y;
        if (!(dn > 0.f)) { d = make_float2(1.f, 0.f); dn = 1.f; }
        const float2 inv = make_float2(d.x / dn, -d.y / dn);
        __syncthreads();
        for (int j = threadIdx.x; j < 2 * b; j += blockDim.x) {
            const float2 v = aug[c][j];
            aug[c][j] = make_float2(v.x * inv.x - v.y * inv.y, v.x * inv.y + v.y * inv.x);
        }
        __syncthreads();
        for (int e = threadIdx.x; e < b * 2 * b; e += blockDim.x) {
            const int r = e / (2 * b), j = e % (2 * b);
            if (r == c) continue;
            const float2 f = aug[r][c], u = aug[c][j];
            if (j == c) continue;  // column c is cleared after the sweep
            aug[r][j] = make_float2(aug[r][j].x - (f.x * u.x - f.y * u.y), aug[r][j].y - (f.x * u.y + f.y * u.x));
        }
        __syncthreads();
        for (int r = threadIdx.x; r < b; r += blockDim.x)
            if (r != c) aug[r][c] = make_float2(0.f, 0.f);
        __syncthreads();
    }
    float2* M = Minv + ((size_t)op * h.nrc + rc) * BJ_MAX * BJ_MAX;
    for (int e = threadIdx.x; e < b * b; e += blockDim.x) {
        const int i = e % b, j = e / b;
        M[(size_t)j * BJ_MAX + i] = aug[i][b + j];
    }
}

// z = blockdiag(D)^-1 q for the systems whose Krylov step is pending.
__global__ void __launch_bounds__(BJ_MAX) hmx_bj_apply_kernel(HmDev h, const float2* __restrict__ Minv, GmBatch bt) {
    const int s = blockIdx.y, rc = blockIdx.x;
    const GmState& st = bt.st[s];
    if (!gm_apply_active(bt, st, MV_Q)) return;
    __shared__ double2 qs[BJ_MAX];
    const GmView g = gm_view(bt, s);
    const double2* qv = bt.Q + g.q + (size_t)st.k * g.n;
    double2* zv = bt.Z + g.q + (size_t)st.k * g.n;
    const int64_t r0 = h.rc_start[rc];
    const int b = (int)(h.rc_start[rc + 1] - r0);
    const int i = threadIdx.x;
    if (i < b) qs[i] = qv[h.perm[r0 + i]];
    __syncthreads();
    if (i >= b) return;
    const float2* M = Minv + ((size_t)(s / h.R) * h.nrc + rc) * BJ_MAX * BJ_MAX;
    double2 acc = make_double2(0, 0);
    for (int j = 0; j < b; ++j) {
        const float2 m = M[(size_t)j * BJ_MAX + i];
        cfma(acc, make_double2(m.x, m.y), qs[j]);
    }
    zv[h.perm[r0 + i]] = acc;
}

}  // namespace

// ---------------------------------------------------------------------------
struct HMixed {
    int64_t n = 0;
    int nops = 0, R = 1, nb = 0, nrc = 0;
    std::vector<HmBlock> blocks;
    std::vector<int32_t> adm_list, rank, diag_blk, rc_ptr, item_blk, item_row;
    std::vector<int64_t> off, toff, rc_start, perm, pos;
    std::vector<double> norms;  // per operator
    int64_t ttot = 0, store_entries = 0, dense_entries = 0, lowrank_entries = 0;
    int64_t nitems = 0, pstride = 0, nchunks = 0;
    DevBuf d_items, d_proj, d_nproj, d_chrc, d_chit, d_rcch, d_part;
    int nsys = 0;
    DevBuf d_blk, d_adm, d_off, d_rank, d_toff, d_store, d_rcs, d_rcp, d_iblk, d_irow, d_perm, d_x, d_t;
    DevBuf d_diag, d_minv, d_small;
    bool bj = false;
    HmDev dev() const {
        HmDev h;
        h.nb = nb;
        h.nadm = (int)adm_list.size();
        h.nrc = nrc;
        h.R = R;
        h.n = n;
        h.ttot = ttot;
        h.blk = d_blk.as<HmBlock>();
        h.adm_list = d_adm.as<int32_t>();
        h.off = d_off.as<int64_t>();
        h.rank = d_rank.as<int32_t>();
        h.toff = d_toff.as<int64_t>();
        h.store = d_store.as<float2>();
        h.rc_start = d_rcs.as<int64_t>();
        h.rc_ptr = d_rcp.as<int32_t>();
        h.item_blk = d_iblk.as<int32_t>();
        h.item_row = d_irow.as<int32_t>();
        h.perm = d_perm.as<int64_t>();
        h.xh = d_x.as<float2>();
        h.xl = h.xh + (size_t)nsys * n;
        h.t = d_t.as<float4>();
        h.items = d_items.as<HmItem>();
        h.nitems = nitems;
        h.proj = d_proj.as<HmProj>();
        h.pstride = pstride;
        h.nproj = d_nproj.as<int32_t>();
        h.ch_rc = d_chrc.as<int32_t>();
        h.ch_it = d_chit.as<int32_t>();
        h.rc_ch = d_rcch.as<int32_t>();
        h.nchunks = nchunks;
        h.part = d_part.as<float4>();
        return h;
    }
};

namespace {
template <class T>
void upload(Context& c, DevBuf& b, const std::vector<T>& v) {
    b.ensure(sizeof(T) * std::max<size_t>(v.size(), 1));
    if (!v.empty()) BEM_CUDA(cudaMemcpyAsync(b.p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, c.stream));
}

void hmx_hook(Context& c, GmWorkspace& ws, int mode, void* user) {
    HMixed& H = *static_cast<HMixed*>(user);
    const HmDev h = H.dev();
    const unsigned ns = (unsigned)ws.bt.nsys;
    hmx_gather_kernel<<<dim3((unsigned)((H.n + 255) / 256), ns), 256, 0, c.stream>>>(h, ws.bt, mode);
    BEM_CHECK_LAUNCH(&c);
    if (h.pstride) {
        const dim3 grid((unsigned)((h.pstride + PJ_WARPS - 1) / PJ_WARPS), ns);
        if (mode == MV_Q) hmx_project_kernel<0><<<grid, PJ_WARPS * 32, 0, c.stream>>>(h, ws.bt, mode);
        else hmx_project_kernel<1><<<grid, PJ_WARPS * 32, 0, c.stream>>>(h, ws.bt, mode);
        BEM_CHECK_LAUNCH(&c);
    }
    const dim3 gr((unsigned)h.nchunks, ns);
    if (mode == MV_Q) hmx_rows_kernel<0><<<gr, RW_THREADS, 0, c.stream>>>(h, ws.bt, mode);
    else hmx_rows_kernel<1><<<gr, RW_THREADS, 0, c.stream>>>(h, ws.bt, mode);
    BEM_CHECK_LAUNCH(&c);
    hmx_reduce_kernel<<<dim3((unsigned)H.nrc, ns), RW_ROWS, 0, c.stream>>>(h, ws.bt, mode);
    BEM_CHECK_LAUNCH(&c);
}

void hmx_bj_hook(Context& c, GmWorkspace& ws, int mode, void* user) {
    (void)mode;
    HMixed& H = *static_cast<HMixed*>(user);
    hmx_bj_apply_kernel<<<dim3((unsigned)H.nrc, (unsigned)ws.bt.nsys), BJ_MAX, 0, c.stream>>>(
        H.dev(), H.d_minv.as<float2>(), ws.bt);
    BEM_CHECK_LAUNCH(&c);
}
}  // namespace

std::shared_ptr<HMixed> hmixed_build(Context& c, Problem& p, int64_t F0, int64_t nops, int R) {
    auto H = std::make_shared<HMixed>();
    const int64_t n = p.n;
    H->n = n;
    H->nops = (int)nops;
    H->R = R;
    H->nsys = (int)(nops * R);
    // cluster order: the leaves of the tree in depth-first order (built once,
    // shared by every frequency)
    std::shared_ptr<void> trees;
    auto F = hmatrix_forest(c, p, &trees);
    H->perm = F->perm;
    H->rc_start.push_back(0);
    for (int32_t v : F->leaves) H->rc_start.push_back(F->nodes[(size_t)v].end);
    require((int64_t)H->perm.size() == n && H->rc_start.back() == n,
            "H-matrix: cluster leaves do not cover the unknowns");
    H->nrc = (int)F->leaves.size();
    H->pos.assign((size_t)n, 0);
    for (int64_t q = 0; q < n; ++q) H->pos[(size_t)H->perm[(size_t)q]] = q;
    DevBuf d_pos;
    upload(c, d_pos, H->pos);
    upload(c, H->d_perm, H->perm);
    const int64_t saved = p.ifreq;
    size_t store_total = 0;
    for (int64_t f = 0; f < nops; ++f) {
        p.ifreq = F0 + f;
        HBuilt B = hmatrix_build_view(c, p, 1, &trees);
        const int nb = (int)B.leaves.size();
        if (f == 0) {
            H->nb = nb;
            H->blocks.resize((size_t)nb);
            for (int b = 0; b < nb; ++b) {
                const HLeafView& L = B.leaves[(size_t)b];
                int64_t r0 = n, c0 = n;
                for (int64_t i = 0; i < L.m; ++i) r0 = std::min(r0, H->pos[(size_t)B.rows[(size_t)(L.row_off + i)]]);
                for (int64_t j = 0; j < L.n; ++j) c0 = std::min(c0, H->pos[(size_t)B.cols[(size_t)(L.col_off + j)]]);
                H->blocks[(size_t)b] = HmBlock{r0, L.m, c0, L.n, L.adm, 0};
                if (L.adm) H->adm_list.push_back(b);
            }
            // per row cluster, the blocks covering it (block order)
            std::vector<std::vector<std::pair<int32_t, int32_t>>> items((size_t)H->nrc);
            std::vector<int> rc_of((size_t)n + 1, 0);
            for (int rc = 0; rc < H->nrc; ++rc)
                for (int64_t q = H->rc_start[(size_t)rc]; q < H->rc_start[(size_t)rc + 1]; ++q) rc_of[(size_t)q] = rc;
            H->diag_blk.assign((size_t)H->nrc, -1);
            for (int b = 0; b < nb; ++b) {
                const HmBlock& K = H->blocks[(size_t)b];
                for (int rc = rc_of[(size_t)K.r0]; rc < H->nrc && H->rc_start[(size_t)rc] < K.r0 + K.m; ++rc) {
                    require(H->rc_start[(size_t)rc + 1] <= K.r0 + K.m && H->rc_start[(size_t)rc] >= K.r0,
                            "H-matrix: a block's rows are not a union of leaf clusters");
                    items[(size_t)rc].emplace_back(b, (int32_t)(H->rc_start[(size_t)rc] - K.r0));
                }
                if (!K.adm && K.m == K.n && K.r0 == K.c0) H->diag_blk[(size_t)rc_of[(size_t)K.r0]] = b;
            }
            H->rc_ptr.push_back(0);
            for (auto& v : items) {
                for (auto& x : v) {
                    H->item_blk.push_back(x.first);
                    H->item_row.push_back(x.second);
                }
                H->rc_ptr.push_back((int32_t)H->item_blk.size());
            }
            H->off.assign((size_t)nops * nb, 0);
            H->rank.assign((size_t)nops * nb, 0);
            H->toff.assign((size_t)nops * nb, 0);
        } else {
            require(nb == H->nb, "H-matrix: block structure differs between frequencies");
        }
        H->norms.push_back(B.norm);
        // offsets of this operator's leaves, then the repack
        std::vector<RepackLeaf> rl((size_t)nb);
        std::vector<int32_t> kmaxs((size_t)nb);
        size_t o = store_total;
        for (int b = 0; b < nb; ++b) {
            const HLeafView& L = B.leaves[(size_t)b];
            const HmBlock& K = H->blocks[(size_t)b];
            const size_t ob = (size_t)f * nb + b;
            H->off[ob] = (int64_t)o;
            H->rank[ob] = L.adm ? L.rank : 0;
            const size_t ent = L.adm ? (size_t)(L.m + L.n) * L.rank : (size_t)L.m * L.n;
            (L.adm ? H->lowrank_entries : H->dense_entries) += (int64_t)ent;
            rl[(size_t)b] = RepackLeaf{L.row_off, L.col_off, L.store_off, (int64_t)o, L.m, L.n, K.r0, K.c0, L.adm,
                                       L.adm ? L.rank : 0};
            kmaxs[(size_t)b] = L.kmax;
            o += ent;
        }
        // grow the FP32 store (keeping the operators already packed)
        if (o * sizeof(float2) > H->d_store.bytes) {
            DevBuf bigger;
            bigger.ensure(std::max<size_t>(o * sizeof(float2), (size_t)(1.25 * (double)H->d_store.bytes)));
            if (store_total)
                BEM_CUDA(cudaMemcpyAsync(bigger.p, H->d_store.p, store_total * sizeof(float2),
                                         cudaMemcpyDeviceToDevice, c.stream));
            c.sync();
            std::swap(bigger.p, H->d_store.p);
            std::swap(bigger.bytes, H->d_store.bytes);
        }
        DevBuf d_rl, d_km;
        upload(c, d_rl, rl);
        upload(c, d_km, kmaxs);
        hmx_repack_kernel<<<(unsigned)nb, 256, 0, c.stream>>>(d_rl.as<RepackLeaf>(), B.d_rows, B.d_cols,
                                                             d_pos.as<int64_t>(), B.d_store, H->d_store.as<float2>());
        BEM_CHECK_LAUNCH(&c);
        hmx_repack_v_kernel<<<(unsigned)nb, 256, 0, c.stream>>>(d_rl.as<RepackLeaf>(), d_km.as<int32_t>(),
                                                               B.d_cols, d_pos.as<int64_t>(), B.d_store,
                                                               H->d_store.as<float2>());
        BEM_CHECK_LAUNCH(&c);
        c.sync();  // the FP64 build is released at the end of this iteration
        store_total = o;
    }
    p.ifreq = saved;
    H->store_entries = (int64_t)store_total;
    // projection offsets: per operator, the admissible blocks' ranks back to back
    int64_t tmax = 0;
    for (int64_t f = 0; f < nops; ++f) {
        int64_t t = 0;
        for (int b : H->adm_list) {
            H->toff[(size_t)f * H->nb + b] = t;
            t += H->rank[(size_t)f * H->nb + b];
        }
        tmax = std::max(tmax, t);
    }
    H->ttot = std::max<int64_t>(tmax, 1);
    // the rows pass: items packed per operator, in chunks of RW_WARPS per cluster
    for (int rc = 0; rc < H->nrc; ++rc)
        require(H->rc_start[(size_t)rc + 1] - H->rc_start[(size_t)rc] <= RW_ROWS,
                "H-matrix mixed form: leaf clusters of more than 64 unknowns");
    H->nitems = (int64_t)H->item_blk.size();
    std::vector<HmItem> items((size_t)(nops * H->nitems));
    for (int64_t f = 0; f < nops; ++f)
        for (int64_t it = 0; it < H->nitems; ++it) {
            const int b = H->item_blk[(size_t)it];
            const HmBlock& K = H->blocks[(size_t)b];
            const size_t ob = (size_t)f * H->nb + b;
            items[(size_t)(f * H->nitems + it)] =
                HmItem{H->off[ob], K.adm ? H->toff[ob] : K.c0, (int32_t)K.m, K.adm ? H->rank[ob] : (int32_t)K.n,
                       H->item_row[(size_t)it], K.adm};
        }
    // chunk c holds items ch_it[c] .. ch_it[c + 1] of one cluster (the
    // clusters' item lists are contiguous, so a cluster's last chunk ends
    // where the next cluster's first begins); a cluster without items still
    // gets one empty chunk, so its rows are written
    std::vector<int32_t> ch_rc, ch_it, rc_ch(1, 0);
    for (int rc = 0; rc < H->nrc; ++rc) {
        const int32_t i0 = H->rc_ptr[(size_t)rc], i1 = H->rc_ptr[(size_t)rc + 1];
        int32_t c0 = i0;
        do {
            ch_rc.push_back(rc);
            ch_it.push_back(c0);
            c0 += RW_WARPS;
        } while (c0 < i1);
        rc_ch.push_back((int32_t)ch_rc.size());
    }
    ch_it.push_back((int32_t)H->nitems);
    H->nchunks = (int64_t)ch_rc.size();
    // the rank columns of every operator's admissible blocks, flat
    std::vector<std::vector<HmProj>> proj((size_t)nops);
    std::vector<int32_t> nproj((size_t)nops);
    for (int64_t f = 0; f < nops; ++f) {
        for (int b : H->adm_list) {
            const HmBlock& K = H->blocks[(size_t)b];
            const size_t ob = (size_t)f * H->nb + b;
            const int r = H->rank[ob];
            for (int k = 0; k < r; k += PJ_COLS)
                proj[(size_t)f].push_back(HmProj{H->off[ob] + K.m * r + (int64_t)k * K.n, K.c0, H->toff[ob] + k,
                                                 (int32_t)K.n, std::min(PJ_COLS, r - k)});
        }
        nproj[(size_t)f] = (int32_t)proj[(size_t)f].size();
        H->pstride = std::max<int64_t>(H->pstride, (int64_t)proj[(size_t)f].size());
    }
    std::vector<HmProj> pflat((size_t)(nops * std::max<int64_t>(H->pstride, 1)));
    for (int64_t f = 0; f < nops; ++f)
        std::copy(proj[(size_t)f].begin(), proj[(size_t)f].end(), pflat.begin() + f * H->pstride);
    upload(c, H->d_items, items);
    upload(c, H->d_proj, pflat);
    upload(c, H->d_nproj, nproj);
    upload(c, H->d_chrc, ch_rc);
    upload(c, H->d_chit, ch_it);
    upload(c, H->d_rcch, rc_ch);
    H->d_part.ensure(sizeof(float4) * (size_t)H->nsys * H->nchunks * RW_ROWS);
    upload(c, H->d_blk, H->blocks);
    upload(c, H->d_adm, H->adm_list);
    upload(c, H->d_off, H->off);
    upload(c, H->d_rank, H->rank);
    upload(c, H->d_toff, H->toff);
    upload(c, H->d_rcs, H->rc_start);
    upload(c, H->d_rcp, H->rc_ptr);
    upload(c, H->d_iblk, H->item_blk);
    upload(c, H->d_irow, H->item_row);
    H->d_x.ensure(sizeof(float2) * 2 * (size_t)H->nsys * n);
    H->d_t.ensure(sizeof(float4) * (size_t)H->nsys * H->ttot);
    c.sync();
    return H;
}

void hmixed_attach(Context& c, GmWorkspace& ws, const std::shared_ptr<HMixed>& H) {
    require(ws.bt.nsys == H->nsys && ws.bt.n == H->n, "H-matrix operator: batch layout mismatch");
    ws.hook = hmx_hook;
    ws.hook_user = H.get();
    // stopping test norms: the H-matrix norm of each system's operator
    std::vector<double> an((size_t)H->nsys);
    for (int s = 0; s < H->nsys; ++s) an[(size_t)s] = H->norms[(size_t)(s / H->R)];
    BEM_CUDA(cudaMemcpyAsync(ws.anorm, an.data(), sizeof(double) * an.size(), cudaMemcpyHostToDevice, c.stream));
    c.sync();
}

bool hmixed_block_jacobi(Context& c, GmWorkspace& ws, const std::shared_ptr<HMixed>& H) {
    for (int rc = 0; rc < H->nrc; ++rc) {
        const int64_t b = H->rc_start[(size_t)rc + 1] - H->rc_start[(size_t)rc];
        if (b > BJ_MAX || H->diag_blk[(size_t)rc] < 0) return false;
    }
    upload(c, H->d_diag, H->diag_blk);
    H->d_minv.ensure(sizeof(float2) * (size_t)H->nops * H->nrc * BJ_MAX * BJ_MAX);
    H->d_small.ensure(sizeof(int));
    BEM_CUDA(cudaMemsetAsync(H->d_small.p, 0, sizeof(int), c.stream));
    BEM_CUDA(cudaFuncSetAttribute(hmx_bj_invert_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)BJ_SMEM));
    hmx_bj_invert_kernel<<<dim3((unsigned)H->nrc, (unsigned)H->nops), 256, BJ_SMEM, c.stream>>>(
        H->dev(), H->d_diag.as<int32_t>(), H->d_minv.as<float2>(), H->d_small.as<int>());
    BEM_CHECK_LAUNCH(&c);
    ws.zb().ensure(sizeof(double2) * gm_q_total(ws));
    ws.bt.Z = ws.zb().as<double2>();
    ws.precond = hmx_bj_hook;
    ws.precond_user = H.get();
    c.sync();
    H->bj = true;
    return true;
}

HMixedStats hmixed_stats(const HMixed& H) {
    HMixedStats s;
    s.blocks = H.nb;
    s.admissible = (int64_t)H.adm_list.size();
    s.clusters = H.nrc;
    s.store_entries = H.store_entries;
    s.dense_entries = H.dense_entries;
    s.lowrank_entries = H.lowrank_entries;
    return s;
}

}  // namespace bem
