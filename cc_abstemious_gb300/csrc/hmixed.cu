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
// system runs in three launches:
//   gather   v_s in cluster order, split into FP32 hi + lo parts;
//   project  t_b = V_b^T v[cols_b] for every admissible block (one CTA per
//            block and system, a warp per rank column);
//   rows     for every leaf row cluster (64 rows), the sum over the blocks that
//            cover it of their dense rows times v[cols] or their U rows times
//            t_b, written back in the original order (one CTA per cluster and
//            system; no atomics, a fixed order).
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
    double2* t;               // nsys x ttot projections
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

// Accumulator of a complex sum of FP32 products with an FP64 operand split
// into hi + lo: EXACT -- every product exact, float-float sums (residuals);
// otherwise FP32 sums of FOLD terms moved into FP64 (Krylov vectors).
constexpr int FOLD = 16;
template <int EXACT>
struct CAcc {
    float rh = 0, rl = 0, ih = 0, il = 0;  // EXACT: float-float; else the open FP32 partial sum in rh, ih
    double dr = 0, di = 0;
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
            rh = fmaf(a.x, xh.x, fmaf(-a.y, xh.y, rh));
            ih = fmaf(a.x, xh.y, fmaf(a.y, xh.x, ih));
            if (++cnt == FOLD) {
                dr += rh;
                di += ih;
                rh = ih = 0.f;
                cnt = 0;
            }
        }
    }
    __device__ __forceinline__ double2 value() const {
        if (EXACT) return make_double2((double)rh + (double)rl, (double)ih + (double)il);
        return make_double2(dr + rh, di + ih);
    }
};

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

template <int EXACT>
__global__ void __launch_bounds__(PJ_WARPS * 32) hmx_project_kernel(HmDev h, GmBatch bt, int mode) {
    const int s = blockIdx.y;
    if (!gm_apply_active(bt, bt.st[s], mode)) return;
    const int b = h.adm_list[blockIdx.x];
    const int op = s / h.R;
    const size_t ob = (size_t)op * h.nb + b;
    const int r = h.rank[ob];
    const HmBlock B = h.blk[b];
    const float2* V = h.store + h.off[ob] + (size_t)B.m * r;
    const float2* xh = h.xh + (size_t)s * h.n + B.c0;
    const float2* xl = h.xl + (size_t)s * h.n + B.c0;
    double2* t = h.t + (size_t)s * h.ttot + h.toff[ob];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int k = warp; k < r; k += PJ_WARPS) {
        const float2* vk = V + (size_t)k * B.n;
        CAcc<EXACT> acc;
        for (int64_t j = lane; j < B.n; j += 32) acc.add(__ldcs(vk + j), xh[j], xl[j]);
        double2 v = acc.value();
        for (int o = 16; o > 0; o >>= 1) {
            v.x += __shfl_down_sync(0xffffffffu, v.x, o);
            v.y += __shfl_down_sync(0xffffffffu, v.y, o);
        }
        if (lane == 0) t[k] = v;
    }
}

constexpr int RW_ROWS = 64, RW_SLICES = 4, RW_THREADS = RW_ROWS * RW_SLICES;

template <int EXACT>
__global__ void __launch_bounds__(RW_THREADS) hmx_rows_kernel(HmDev h, GmBatch bt, int mode) {
    const int s = blockIdx.y;
    if (!gm_apply_active(bt, bt.st[s], mode)) return;
    __shared__ double2 red[RW_SLICES][RW_ROWS];
    const int rc = blockIdx.x, op = s / h.R;
    const int q = threadIdx.x / RW_ROWS;
    const int64_t rs = h.rc_start[rc];
    const int rows = (int)(h.rc_start[rc + 1] - rs);
    const float2* xh = h.xh + (size_t)s * h.n;
    const float2* xl = h.xl + (size_t)s * h.n;
    const double2* tsys = h.t + (size_t)s * h.ttot;
    const GmView g = gm_view(bt, s);
    // clusters of up to RW_ROWS rows take one pass (leaf size <= 64)
    for (int i0 = 0; i0 < rows; i0 += RW_ROWS) {
        const int i = i0 + threadIdx.x % RW_ROWS;
        CAcc<EXACT> acc;
        if (i < rows) {
            for (int it = h.rc_ptr[rc]; it < h.rc_ptr[rc + 1]; ++it) {
                const int b = h.item_blk[it];
                const int64_t lr = h.item_row[it] + i;
                const size_t ob = (size_t)op * h.nb + b;
                const HmBlock B = h.blk[b];
                const float2* D = h.store + h.off[ob];
                if (!B.adm) {
                    for (int64_t j = q; j < B.n; j += RW_SLICES)
                        acc.add(__ldcs(D + (size_t)j * B.m + lr), xh[B.c0 + j], xl[B.c0 + j]);
                } else {
                    const int r = h.rank[ob];
                    const double2* t = tsys + h.toff[ob];
                    for (int k = q; k < r; k += RW_SLICES) {
                        const double2 tk = t[k];
                        const float thx = (float)tk.x, thy = (float)tk.y;
                        acc.add(__ldcs(D + (size_t)k * B.m + lr), make_float2(thx, thy),
                                make_float2((float)(tk.x - (double)thx), (float)(tk.y - (double)thy)));
                    }
                }
            }
        }
        red[q][threadIdx.x % RW_ROWS] = acc.value();
        __syncthreads();
        if (q == 0 && i < rows) {
            double2 v = red[0][i - i0];
            for (int u = 1; u < RW_SLICES; ++u) {
                v.x += red[u][i - i0].x;
                v.y += red[u][i - i0].y;
            }
            bt.W[g.v + h.perm[rs + i]] = v;
        }
        __syncthreads();
    }
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
        h.t = d_t.as<double2>();
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
    if (h.nadm) {
        if (mode == MV_Q) hmx_project_kernel<0><<<dim3((unsigned)h.nadm, ns), PJ_WARPS * 32, 0, c.stream>>>(h, ws.bt, mode);
        else hmx_project_kernel<1><<<dim3((unsigned)h.nadm, ns), PJ_WARPS * 32, 0, c.stream>>>(h, ws.bt, mode);
        BEM_CHECK_LAUNCH(&c);
    }
    if (mode == MV_Q) hmx_rows_kernel<0><<<dim3((unsigned)H.nrc, ns), RW_THREADS, 0, c.stream>>>(h, ws.bt, mode);
    else hmx_rows_kernel<1><<<dim3((unsigned)H.nrc, ns), RW_THREADS, 0, c.stream>>>(h, ws.bt, mode);
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
    // cluster order: the leaves of the tree in depth-first order
    auto leaves = cluster_leaves(p.cpts, 8, p.in.hm_leaf);
    H->perm.reserve((size_t)n);
    H->rc_start.push_back(0);
    for (auto& l : leaves) {
        H->perm.insert(H->perm.end(), l.idx.begin(), l.idx.end());
        H->rc_start.push_back((int64_t)H->perm.size());
    }
    require((int64_t)H->perm.size() == n, "H-matrix: cluster leaves do not cover the unknowns");
    H->nrc = (int)leaves.size();
    H->pos.assign((size_t)n, 0);
    for (int64_t q = 0; q < n; ++q) H->pos[(size_t)H->perm[(size_t)q]] = q;
    DevBuf d_pos;
    upload(c, d_pos, H->pos);
    upload(c, H->d_perm, H->perm);
    const int64_t saved = p.ifreq;
    size_t store_total = 0;
    std::shared_ptr<void> trees;  // built once, shared by every frequency
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
    H->d_t.ensure(sizeof(double2) * (size_t)H->nsys * H->ttot);
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
