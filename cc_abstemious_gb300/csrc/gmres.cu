// Restarted GMRES (gmres.rs:35-202) as a device-side state machine over a
// batch of independent systems: of equal size n (uniform layout), or of
// different sizes (ragged layout, per-system offsets in GmSys).
//
// One iteration is the fixed launch sequence
//   apply(START) -> start -> apply(Q) -> [Gram-Schmidt x 2] -> arnoldi -> apply(CHECK) -> check
// where every kernel reads the per-system state and returns immediately when
// it has nothing to do.  The sequence can therefore be issued step by step
// (plain form, host reads the state after each step) or captured into a CUDA
// graph covering several iterations of every system (batched form).
//
// Operator: FP64 matrix (plain form, bit-for-bit the reference arithmetic up
// to summation order) or FP32 matrix with FP64 vectors and compensated
// products/sums (mixed form).  Arnoldi, Givens rotations, the small
// triangular solve and the stopping test are FP64: the reference form keeps
// its single-CTA modified Gram-Schmidt, the mixed and refined forms
// orthogonalise across the whole GPU (classical Gram-Schmidt twice).
#include <mutex>

#include "common.cuh"
#include "complex.cuh"
#include "gmres.cuh"

namespace bem {

constexpr int MV_ROWS_PER_THREAD = 2;
constexpr int MV_THREADS = 256;
constexpr int MV_ROWS = MV_ROWS_PER_THREAD * MV_THREADS;  // 512
constexpr int MV_COLS = 512;
constexpr int AR_THREADS = 1024;
// largest Krylov vector kept in the Arnoldi kernel's shared memory (n <= 12800)
constexpr size_t AR_SMEM_CAP = 200 * 1024;

__device__ __forceinline__ bool mv_active(const GmState& s, int mode) {
    if (s.done) return false;
    if (mode == MV_START) return s.need_start != 0;
    if (mode == MV_Q) return s.need_start == 0 && s.check == 0;
    return s.check != 0;  // MV_CHECK
}

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// acc (hi, lo) += a * b with a*b = p + e exactly (FMA) and a small extra term.
__device__ __forceinline__ void ff_acc(float& hi, float& lo, float a, float b) {
    float p = a * b;
    float e = fmaf(a, b, -p);
    float s, err;
    two_sum(hi, p, s, err);
    hi = s;
    lo += err + e;
}

// Batched operator application W_s = A_s v_s, v_s = x_s (START/CHECK) or
// Q_s[:, k] (Q).  Grid (row blocks, column chunks, systems); partial sums of
// the column chunks are reduced in a fixed order by the last CTA of each row
// block (ticket counter, no waiting).  Each thread owns two consecutive rows
// and streams its columns with 16-byte loads, eight columns in flight.
//
// FP32 operators, two accumulation schemes:
//  EXACT (true residuals, START/CHECK): x split into hi + lo floats, every
//        product split exactly with an FMA and summed in float-float;
//  FAST  (Krylov vectors, Q): FP32 sums of 8 columns folded into a float-float
//        accumulator; ~1e-7 relative, which only perturbs the Krylov basis:
//        the exact residual at each check and restart keeps the answer exact.
// Split FP64 operators (EXACT == 2, every mode): the EXACT scheme over the
// FP32 matrix plus the products of its remainder plane with x's hi part, so
// the mat-vec carries the FP64 operator to ~2^-44 on the FP32 pipe (GB300's
// FP64 rate is 1/64 of it) while streaming the same 16 B per entry.
constexpr int MV_UNROLL = 8;

template <typename T, int EXACT, int U = MV_UNROLL>
__global__ void __launch_bounds__(MV_THREADS) gm_apply_kernel(GmBatch bt, int mode) {
    static_assert(MV_COLS % U == 0, "the column chunk is a whole number of unrolled groups");
    int s, bx, by;
    if (bt.sys) {
        // ragged batch: one flattened grid over every system's (row block,
        // column chunk) tiles; the system is found by bisection on tile0
        const int64_t t = blockIdx.x;
        int lo = 0, hi = bt.nsys - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (bt.sys[mid].tile0 <= t) lo = mid;
            else hi = mid - 1;
        }
        s = lo;
        const int64_t local = t - bt.sys[s].tile0;
        const int rbs = bt.sys[s].rb;
        bx = (int)(local % rbs);
        by = (int)(local / rbs);
    } else {
        s = blockIdx.z;
        bx = blockIdx.x;
        by = blockIdx.y;
    }
    GmState& st = bt.st[s];
    if (!mv_active(st, mode)) return;
    // outside the reference-faithful mode the first cycle starts from x = 0,
    // so its residual is b itself: no product needed
    if (mode == MV_START && !bt.ref_dotc && st.restarts == 0) return;
    const GmView g = gm_view(bt, s);
    const int64_t n = g.n;
    const double2* kv = bt.Z ? bt.Z : bt.Q;  // right preconditioning applies A to M q_k
    const double2* v = (mode == MV_Q) ? kv + g.q + (size_t)st.k * n : bt.X + g.v;
    __shared__ float2 xh[MV_COLS], xl[MV_COLS];
    __shared__ double2 xd[MV_COLS];
    __shared__ int last;
    const int64_t j0 = (int64_t)by * MV_COLS;
    const int jn = (int)min((int64_t)MV_COLS, n - j0);
    for (int t = threadIdx.x; t < MV_COLS; t += MV_THREADS) {
        double2 x = t < jn ? v[j0 + t] : make_double2(0, 0);
        if (sizeof(T) == sizeof(float2)) {
            float hx = (float)x.x, hy = (float)x.y;
            xh[t] = make_float2(hx, hy);
            xl[t] = make_float2((float)(x.x - (double)hx), (float)(x.y - (double)hy));
        } else {
            xd[t] = x;
        }
    }
    __syncthreads();
    const int64_t i0 = (int64_t)bx * MV_ROWS + MV_ROWS_PER_THREAD * threadIdx.x;
    const int64_t lda = g.lda;
    double2 r0 = make_double2(0, 0), r1 = make_double2(0, 0);
    if (i0 < n) {
        const bool pair = (i0 + 1 < n);
        if (sizeof(T) == sizeof(float2)) {
            const float2* A = reinterpret_cast<const float2*>(bt.A) + g.a + i0;
            // float-float accumulators for (re0, im0, re1, im1)
            float h0 = 0, l0 = 0, h1 = 0, l1 = 0, h2 = 0, l2 = 0, h3 = 0, l3 = 0;
            for (int q0 = 0; q0 < jn; q0 += U) {
                float4 a[U], z[EXACT == 2 ? U : 1];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const int q = q0 + u;
                    if (q < jn) {
                        const float2* col = A + (j0 + q) * lda;
                        if (pair) a[u] = __ldcs(reinterpret_cast<const float4*>(col));
                        else { float2 t = col[0]; a[u] = make_float4(t.x, t.y, 0.f, 0.f); }
                        if (EXACT == 2) {
                            const float2* cl = col + bt.split_lo;
                            if (pair) z[u] = __ldcs(reinterpret_cast<const float4*>(cl));
                            else { float2 t = cl[0]; z[u] = make_float4(t.x, t.y, 0.f, 0.f); }
                        }
                    } else {
                        a[u] = make_float4(0.f, 0.f, 0.f, 0.f);
                        if (EXACT == 2) z[u] = make_float4(0.f, 0.f, 0.f, 0.f);
                    }
                }
                if (EXACT) {
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        const float2 H = xh[q0 + u], L = xl[q0 + u];
                        const float4 w = a[u];
                        ff_acc(h0, l0, w.x, H.x); ff_acc(h0, l0, -w.y, H.y);
                        ff_acc(h1, l1, w.x, H.y); ff_acc(h1, l1, w.y, H.x);
                        ff_acc(h2, l2, w.z, H.x); ff_acc(h2, l2, -w.w, H.y);
                        ff_acc(h3, l3, w.z, H.y); ff_acc(h3, l3, w.w, H.x);
                        l0 = fmaf(w.x, L.x, fmaf(-w.y, L.y, l0));
                        l1 = fmaf(w.x, L.y, fmaf(w.y, L.x, l1));
                        l2 = fmaf(w.z, L.x, fmaf(-w.w, L.y, l2));
                        l3 = fmaf(w.z, L.y, fmaf(w.w, L.x, l3));
                        if (EXACT == 2) {
                            const float4 y = z[EXACT == 2 ? u : 0];
                            l0 = fmaf(y.x, H.x, fmaf(-y.y, H.y, l0));
                            l1 = fmaf(y.x, H.y, fmaf(y.y, H.x, l1));
                            l2 = fmaf(y.z, H.x, fmaf(-y.w, H.y, l2));
                            l3 = fmaf(y.z, H.y, fmaf(y.w, H.x, l3));
                        }
                    }
                } else {
                    float b0 = 0, b1 = 0, b2 = 0, b3 = 0;
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        const float2 H = xh[q0 + u];
                        const float4 w = a[u];
                        b0 = fmaf(w.x, H.x, fmaf(-w.y, H.y, b0));
                        b1 = fmaf(w.x, H.y, fmaf(w.y, H.x, b1));
                        b2 = fmaf(w.z, H.x, fmaf(-w.w, H.y, b2));
                        b3 = fmaf(w.z, H.y, fmaf(w.w, H.x, b3));
                    }
                    float e, t;
                    two_sum(h0, b0, t, e); h0 = t; l0 += e;
                    two_sum(h1, b1, t, e); h1 = t; l1 += e;
                    two_sum(h2, b2, t, e); h2 = t; l2 += e;
                    two_sum(h3, b3, t, e); h3 = t; l3 += e;
                }
            }
            r0 = make_double2((double)h0 + (double)l0, (double)h1 + (double)l1);
            r1 = make_double2((double)h2 + (double)l2, (double)h3 + (double)l3);
        } else {
            const double2* A = reinterpret_cast<const double2*>(bt.A) + g.a + i0;
            for (int q0 = 0; q0 < jn; q0 += U) {
                double2 a0[U], a1[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const int q = q0 + u;
                    const double2* col = A + (j0 + (q < jn ? q : 0)) * lda;
                    a0[u] = q < jn ? col[0] : make_double2(0, 0);
                    a1[u] = (q < jn && pair) ? col[1] : make_double2(0, 0);
                }
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const double2 xv = xd[q0 + u];
                    cfma(r0, a0[u], xv);
                    cfma(r1, a1[u], xv);
                }
            }
        }
        double2* part = bt.part + g.p + (size_t)by * g.n_pad;
        part[i0] = r0;
        if (pair) part[i0 + 1] = r1;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        int* tk = bt.tickets + g.t + bx;
        last = (atomicAdd(tk, 1) == g.cb - 1);
        if (last) *tk = 0;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double2* W = bt.W + g.v;
    for (int rr = 0; rr < MV_ROWS_PER_THREAD; ++rr) {
        int64_t i = i0 + rr;
        if (i >= n) break;
        double2 acc = make_double2(0, 0);
        const double2* part = bt.part + g.p;
        for (int c = 0; c < g.cb; ++c) acc = cadd(acc, part[(size_t)c * g.n_pad + i]);
        W[i] = acc;
    }
}

// ---------------------------------------------------------------------------
// Block-wide FP64 reductions (1024 threads).
__device__ __forceinline__ double block_sum(double v, double* sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    if (w == 0) {
        v = l < (int)(blockDim.x >> 5) ? sh[l] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (l == 0) sh[32] = v;
    }
    __syncthreads();
    return sh[32];
}

__device__ __forceinline__ double2 block_sum2(double2 v, double* sh) {
    for (int o = 16; o > 0; o >>= 1) {
        v.x += __shfl_down_sync(0xffffffffu, v.x, o);
        v.y += __shfl_down_sync(0xffffffffu, v.y, o);
    }
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) { sh[2 * w] = v.x; sh[2 * w + 1] = v.y; }
    __syncthreads();
    if (w == 0) {
        int nw = blockDim.x >> 5;
        v.x = l < nw ? sh[2 * l] : 0.0;
        v.y = l < nw ? sh[2 * l + 1] : 0.0;
        for (int o = 16; o > 0; o >>= 1) {
            v.x += __shfl_down_sync(0xffffffffu, v.x, o);
            v.y += __shfl_down_sync(0xffffffffu, v.y, o);
        }
        if (l == 0) { sh[64] = v.x; sh[65] = v.y; }
    }
    __syncthreads();
    return make_double2(sh[64], sh[65]);
}

__device__ double vec_norm(const double2* v, int64_t n, double* sh) {
    double s = 0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s += v[i].x * v[i].x + v[i].y * v[i].y;
    return sqrt(block_sum(s, sh));
}

// Cycle start (gmres.rs:84-106): r = b - A x, q_0 = r / ||r||, beta_0 = ||r||.
__global__ void __launch_bounds__(AR_THREADS) gm_start_kernel(GmBatch bt) {
    const int s = blockIdx.x;
    GmState& st = bt.st[s];
    if (st.done || !st.need_start) return;
    __shared__ double sh[80];
    const GmView g = gm_view(bt, s);
    const int64_t n = g.n;
    const double2* b = bt.B + g.v;
    const double2* W = bt.W + g.v;
    double2* Q = bt.Q + g.q;
    const bool zero_x = !bt.ref_dotc && st.restarts == 0;  // x = 0: A x not formed
    double acc = 0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        double2 r = zero_x ? b[i] : csub(b[i], W[i]);
        Q[i] = r;
        acc += r.x * r.x + r.y * r.y;
    }
    double rn = sqrt(block_sum(acc, sh));
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        double2 r = Q[i];
        Q[i] = make_double2(r.x / rn, r.y / rn);
    }
    double xn = vec_norm(bt.X + g.v, n, sh);
    if (threadIdx.x == 0) {
        GmSmall sm = gm_small(bt, s);
        for (int i = 0; i <= bt.m; ++i) sm.beta[i] = make_double2(0, 0);
        for (int i = 0; i < bt.m; ++i) { sm.cs[i] = make_double2(0, 0); sm.sn[i] = make_double2(0, 0); }
        sm.beta[0] = make_double2(rn, 0.0);
        st.xnorm = xn;
        st.error = rn / (st.anorm * xn + st.bnorm);
        st.k = 0;
        st.need_start = 0;
        st.check = 0;
        st.num_mv += zero_x ? 0 : 1;
    }
}

// ---------------------------------------------------------------------------
// Gram-Schmidt of the mixed and refined forms across the whole GPU: classical
// Gram-Schmidt applied twice (the second pass re-orthogonalises; as accurate
// as the modified form), in FP64.  Every CTA owns a chunk of GS_ROWS rows of
// one system: the dots kernel forms its chunk's contribution to q_i^H w for
// every i <= k (a warp per basis vector), the update kernel adds the chunks'
// contributions in chunk order and subtracts Q h from its rows (and, after
// the second pass, leaves the squared norm of its rows).  Systems pending a
// Krylov step only (the Arnoldi kernel's predicate).
constexpr int GS_ROWS = 512, GS_THREADS = 256;

__device__ __forceinline__ bool gm_arnoldi_active(const GmState& st) {
    return !(st.done || st.need_start || st.check);
}

__global__ void __launch_bounds__(GS_THREADS) gm_gs_dots_kernel(GmBatch bt) {
    const int s = blockIdx.y, c = blockIdx.x;
    const GmState& st = bt.st[s];
    if (!gm_arnoldi_active(st)) return;
    const GmView g = gm_view(bt, s);
    const int64_t r0 = (int64_t)c * GS_ROWS;
    if (r0 >= g.n) return;
    const int rows = (int)min((int64_t)GS_ROWS, g.n - r0);
    __shared__ double2 ws[GS_ROWS];
    const double2* W = bt.W + g.v + r0;
    for (int l = threadIdx.x; l < rows; l += GS_THREADS) ws[l] = W[l];
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const double2* Q = bt.Q + g.q + r0;
    double2* part = bt.gs_part + ((size_t)s * bt.gs_chunks + c) * (bt.m + 1);
    for (int i = warp; i <= st.k; i += GS_THREADS / 32) {
        const double2* qi = Q + (size_t)i * g.n;
        double2 acc = make_double2(0, 0);
        for (int l = lane; l < rows; l += 32) cfma(acc, cconj(qi[l]), ws[l]);
        for (int o = 16; o > 0; o >>= 1) {
            acc.x += __shfl_down_sync(0xffffffffu, acc.x, o);
            acc.y += __shfl_down_sync(0xffffffffu, acc.y, o);
        }
        if (lane == 0) part[i] = acc;
    }
}

// pass 0: hk1[i] = h_i; pass 1: hk1[i] += h_i and the chunk's squared norm.
__global__ void __launch_bounds__(GS_THREADS) gm_gs_update_kernel(GmBatch bt, int pass) {
    const int s = blockIdx.y, c = blockIdx.x;
    const GmState& st = bt.st[s];
    if (!gm_arnoldi_active(st)) return;
    const GmView g = gm_view(bt, s);
    const int64_t r0 = (int64_t)c * GS_ROWS;
    if (r0 >= g.n) return;
    const int rows = (int)min((int64_t)GS_ROWS, g.n - r0);
    const int k = st.k;
    const int nch = (int)((g.n + GS_ROWS - 1) / GS_ROWS);
    extern __shared__ double2 hsum[];  // k + 1 coefficients
    __shared__ double red[GS_THREADS / 32];
    const double2* part = bt.gs_part + (size_t)s * bt.gs_chunks * (bt.m + 1);
    for (int i = threadIdx.x; i <= k; i += GS_THREADS) {
        double2 h = make_double2(0, 0);
        for (int cc = 0; cc < nch; ++cc) h = cadd(h, part[(size_t)cc * (bt.m + 1) + i]);
        hsum[i] = h;
    }
    __syncthreads();
    if (c == 0 && threadIdx.x == 0) {
        GmSmall sm = gm_small(bt, s);
        for (int i = 0; i <= k; ++i) sm.hk1[i] = pass == 0 ? hsum[i] : cadd(sm.hk1[i], hsum[i]);
    }
    double2* W = bt.W + g.v + r0;
    const double2* Q = bt.Q + g.q + r0;
    double nn = 0;
    for (int l = threadIdx.x; l < rows; l += GS_THREADS) {
        double2 a = W[l];
        for (int i = 0; i <= k; ++i) cfma(a, cneg(hsum[i]), Q[(size_t)i * g.n + l]);
        W[l] = a;
        nn += a.x * a.x + a.y * a.y;
    }
    if (pass == 1) {
        for (int o = 16; o > 0; o >>= 1) nn += __shfl_down_sync(0xffffffffu, nn, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = nn;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0;
            for (int w = 0; w < GS_THREADS / 32; ++w) t += red[w];
            bt.gs_norm[(size_t)s * bt.gs_chunks + c] = t;
        }
    }
}

// Arnoldi step k with modified Gram-Schmidt (gmres.rs:158-176), Givens
// update (gmres.rs:178-202), residual estimate and, when the estimate passes
// or the cycle ends, the solution update x += Q_k H_k^{-1} beta_k
// (gmres.rs:146-157).  The Krylov vector w lives in shared memory when it
// fits (`w_in_smem`), else in the W buffer.
__global__ void __launch_bounds__(AR_THREADS) gm_arnoldi_kernel(GmBatch bt, int w_in_smem) {
    const int s = blockIdx.x;
    GmState& st = bt.st[s];
    if (st.done || st.need_start || st.check) return;
    extern __shared__ double2 wsh[];
    __shared__ double sh[80];
    __shared__ double2 hsh;
    const GmView g = gm_view(bt, s);
    const int64_t n = g.n;
    const int k = st.k;
    const int m = bt.m;
    double2* Q = bt.Q + g.q;
    double2* Wg = bt.W + g.v;
    double2* w = w_in_smem ? wsh : Wg;
    GmSmall sm = gm_small(bt, s);
    double2* qk1 = Q + (size_t)(k + 1) * n;
    double hn;
    if (bt.gs_part && !bt.ref_dotc) {
        // orthogonalised across the GPU (gm_gs_dots_kernel /
        // gm_gs_update_kernel): h_{:,k} is in hk1[0..k], w in W; its norm
        // from the chunks' partial squares
        double nn = 0;
        const int nch = (int)((n + GS_ROWS - 1) / GS_ROWS);  // this system's chunks (ragged batches)
        for (int c = 0; c < nch; ++c) nn += bt.gs_norm[(size_t)s * bt.gs_chunks + c];
        hn = sqrt(nn);
        const double sc = 1.0 / hn;
        for (int64_t l = threadIdx.x; l < n; l += blockDim.x) {
            const double2 a = Wg[l];
            qk1[l] = make_double2(a.x * sc, a.y * sc);
        }
    } else {
        if (w_in_smem)
            for (int64_t i = threadIdx.x; i < n; i += blockDim.x) w[i] = Wg[i];
        __syncthreads();
        // modified Gram-Schmidt
        for (int i = 0; i <= k; ++i) {
            const double2* qi = Q + (size_t)i * n;
            double2 acc = make_double2(0, 0);
            for (int64_t l = threadIdx.x; l < n; l += blockDim.x) {
                double2 a = w[l], q = qi[l];
                if (bt.ref_dotc) cfma(acc, cconj(a), q);  // nalgebra dotc(qk1, q_i) = sum conj(qk1) q_i
                else cfma(acc, cconj(q), a);             // q_i^H w
            }
            double2 h = block_sum2(acc, sh);
            for (int64_t l = threadIdx.x; l < n; l += blockDim.x) {
                double2 a = w[l];
                cfma(a, cneg(h), qi[l]);
                w[l] = a;
            }
            if (threadIdx.x == 0) sm.hk1[i] = h;
            __syncthreads();
        }
        hn = vec_norm(w, n, sh);
        // scale = 1 / hk1[k+1] as a complex division (gmres.rs:172)
        double2 scale = cdiv(make_double2(1.0, 0.0), make_double2(hn, 0.0));
        for (int64_t l = threadIdx.x; l < n; l += blockDim.x) qk1[l] = cmul(w[l], scale);
    }
    if (threadIdx.x == 0) {
        sm.hk1[k + 1] = make_double2(hn, 0.0);
        // apply previous rotations
        for (int i = 0; i < k; ++i) {
            double2 t = cadd(cmul(sm.cs[i], sm.hk1[i]), cmul(sm.sn[i], sm.hk1[i + 1]));
            sm.hk1[i + 1] = cadd(cmul(cneg(cconj(sm.sn[i])), sm.hk1[i]), cmul(sm.cs[i], sm.hk1[i + 1]));
            sm.hk1[i] = t;
        }
        // new rotation (LAWN 148)
        double2 v1 = sm.hk1[k], v2 = sm.hk1[k + 1];
        double a1 = cabs_(v1);
        double2 signf = (v1.x == 0.0 && v1.y == 0.0) ? make_double2(1.0, 0.0) : make_double2(v1.x / a1, v1.y / a1);
        double r = sqrt(cnorm2(v1) + cnorm2(v2));
        double2 cs = make_double2(a1 / r, 0.0);
        double2 sn = cmul(signf, cconj(v2));
        sn = make_double2(sn.x / r, sn.y / r);
        sm.cs[k] = cs;
        sm.sn[k] = sn;
        sm.hk1[k] = cadd(cmul(cs, sm.hk1[k]), cmul(sn, sm.hk1[k + 1]));
        sm.hk1[k + 1] = make_double2(0, 0);
        for (int i = 0; i < k + 2; ++i) sm.H[(size_t)k * (m + 1) + i] = sm.hk1[i];
        sm.beta[k + 1] = cmul(cneg(cconj(sn)), sm.beta[k]);
        sm.beta[k] = cmul(sm.beta[k], cs);
        st.error = cabs_(sm.beta[k + 1]) / (st.anorm * st.xnorm + st.bnorm);
        st.num_mv += 1;
        st.iterations += 1;
        int chk = (st.error < st.tol) || (k == st.m - 1);
        st.check = chk;
        if (chk) {
            // y = H_k^{-1} beta_k: H_k is upper triangular after the rotations
            for (int i = k; i >= 0; --i) {
                double2 v = sm.beta[i];
                for (int q = i + 1; q <= k; ++q) v = csub(v, cmul(sm.H[(size_t)q * (m + 1) + i], sm.y[q]));
                sm.y[i] = cdiv(v, sm.H[(size_t)i * (m + 1) + i]);
            }
        } else {
            st.k = k + 1;
        }
        hsh.x = chk;
    }
    __syncthreads();
    if (hsh.x != 0.0) {
        // x += Q_k y, or Z_k y with flexible right preconditioning
        double2* x = bt.X + g.v;
        const double2* Zs = bt.Z ? bt.Z + g.q : Q;
        for (int64_t l = threadIdx.x; l < n; l += blockDim.x) {
            double2 a = x[l];
            for (int j = 0; j <= k; ++j) cfma(a, Zs[(size_t)j * n + l], sm.y[j]);
            x[l] = a;
        }
    }
}

// True residual check (gmres.rs:122-138).
__global__ void __launch_bounds__(AR_THREADS) gm_check_kernel(GmBatch bt) {
    const int s = blockIdx.x;
    GmState& st = bt.st[s];
    if (st.done || !st.check) return;
    __shared__ double sh[80];
    const GmView g = gm_view(bt, s);
    const int64_t n = g.n;
    const double2* b = bt.B + g.v;
    const double2* W = bt.W + g.v;
    double acc = 0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        double2 r = csub(b[i], W[i]);
        acc += r.x * r.x + r.y * r.y;
    }
    double rn = sqrt(block_sum(acc, sh));
    double xn = vec_norm(bt.X + g.v, n, sh);
    if (threadIdx.x == 0) {
        st.num_mv += 1;
        st.xnorm = xn;
        st.error = rn / (st.anorm * xn + st.bnorm);
        st.check = 0;
        if (st.error < st.tol) {
            st.done = 1;
            st.converged = 1;
        } else if (st.k == st.m - 1 || !bt.ref_dotc) {
            // End of the cycle.  Outside the reference-faithful mode a failed
            // check also restarts from the updated x (an iterative-refinement
            // step), instead of continuing the Arnoldi process and adding the
            // Krylov correction to x a second time at the next check.
            st.restarts += 1;
            if (st.restarts >= st.max_restarts) st.done = 1;
            else st.need_start = 1;
        } else {
            st.k += 1;
        }
    }
}

// Zero initial guess and the per-system constants.
__global__ void gm_init_kernel(GmBatch bt, const double* anorm, double tol, int64_t max_restarts,
                               const double* __restrict__ tols, const int64_t* __restrict__ maxrs,
                               const int* __restrict__ ms) {
    const int s = blockIdx.x;
    __shared__ double sh[80];
    const GmView g = gm_view(bt, s);
    const int64_t n = g.n;
    double2* x = bt.X + g.v;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) x[i] = make_double2(0, 0);
    double bn = vec_norm(bt.B + g.v, n, sh);
    if (threadIdx.x == 0) {
        GmState& st = bt.st[s];
        st.anorm = anorm[s];
        st.bnorm = bn;
        st.tol = tols ? tols[s] : tol;
        st.m = ms ? ms[s] : bt.m;
        st.xnorm = 0;
        st.error = 1.0;
        st.k = 0;
        st.need_start = 1;
        st.check = 0;
        st.done = 0;
        st.converged = 0;
        st.num_mv = 0;
        st.iterations = 0;
        st.restarts = 0;
        st.max_restarts = maxrs ? maxrs[s] : max_restarts;
        if (bn == 0.0) {  // zero right-hand side: x = 0 is exact
            st.done = 1;
            st.converged = 1;
            st.error = 0;
        }
    }
}

// Frobenius norms of a batch of matrices (FP64 or FP32 entries): CTAs stride
// over columns, threads over rows (coalesced, no index division).
template <typename T>
__global__ void batch_frob_kernel(const void* A, int64_t n, int64_t lda, size_t mat_stride, double* part, int nb) {
    __shared__ double sh[80];
    int s = blockIdx.y;
    const T* M = reinterpret_cast<const T*>(A) + (size_t)s * mat_stride;
    double acc = 0;
    for (int64_t j = blockIdx.x; j < n; j += gridDim.x) {
        const T* col = M + j * lda;
        for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
            T v = col[i];
            acc += (double)v.x * (double)v.x + (double)v.y * (double)v.y;
        }
    }
    double r = block_sum(acc, sh);
    if (threadIdx.x == 0) part[(size_t)s * nb + blockIdx.x] = r;
}

__global__ void finish_norms_kernel(const double* part, int nb, int nsys, double* out) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsys) return;
    double acc = 0;
    for (int b = 0; b < nb; ++b) acc += part[(size_t)s * nb + b];
    out[s] = sqrt(acc);
}

// ---------------------------------------------------------------------------
// The Arnoldi kernel keeps w in dynamic shared memory when it fits
// (n * 16 B <= AR_SMEM_CAP).  The kernel attribute is process-wide, so it is
// raised once per device to the cap and never lowered: a smaller solve on
// another thread cannot shrink the limit under a larger one's launch or graph.
namespace {
constexpr int AR_MAX_DEVICES = 64;
std::once_flag g_ar_smem_once[AR_MAX_DEVICES];
}  // namespace

void arnoldi_allow_smem(int device) {
    require(device >= 0 && device < AR_MAX_DEVICES, "device index out of range");
    // a failed set throws out of call_once, which leaves the flag unset so the
    // next call tries again
    std::call_once(g_ar_smem_once[device], [] {
        cudaError_t err = cudaFuncSetAttribute(gm_arnoldi_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)AR_SMEM_CAP);
        if (err != cudaSuccess)
            throw Error(BEM_ERR_CUDA,
                        std::string("cudaFuncSetAttribute(gm_arnoldi_kernel): ") + cudaGetErrorString(err));
    });
}

GmWorkspace::~GmWorkspace() {
    if (graph_exec) cudaGraphExecDestroy(graph_exec);
}

void gm_prepare(Context& ctx, GmWorkspace& ws, int nsys, int64_t n, int m, const void* A, int64_t lda,
                size_t mat_stride, bool fp32, bool ref_dotc) {
    GmBatch& bt = ws.bt;
    bt.nsys = nsys;
    bt.n = n;
    bt.n_pad = (n + MV_ROWS - 1) / MV_ROWS * MV_ROWS;
    bt.m = m;
    bt.A = A;
    bt.lda = lda;
    bt.mat_stride = mat_stride;
    bt.ref_dotc = ref_dotc ? 1 : 0;
    bt.qstride = (size_t)n * (m + 1);
    ws.fp32 = fp32;
    int rb = (int)((n + MV_ROWS - 1) / MV_ROWS), cb = (int)((n + MV_COLS - 1) / MV_COLS);
    ws.rb = rb;
    ws.cb = cb;
    bt.rb = rb;
    bt.cb = cb;
    bt.sys = nullptr;
    bt.ntiles = 0;
    ws.sys_host.clear();
    size_t small = gm_small_size(m);
    size_t bytes = 0;
    auto carve = [&](size_t b) { size_t o = bytes; bytes += (b + 255) / 256 * 256; return o; };
    size_t oX = carve(sizeof(double2) * nsys * n), oB = carve(sizeof(double2) * nsys * n);
    size_t oQ = carve(sizeof(double2) * nsys * bt.qstride), oW = carve(sizeof(double2) * nsys * n);
    size_t oP = carve(sizeof(double2) * nsys * cb * bt.n_pad), oT = carve(sizeof(int) * nsys * rb);
    size_t oS = carve(sizeof(double2) * nsys * small), oSt = carve(sizeof(GmState) * nsys);
    size_t oN = carve(sizeof(double) * nsys * 1024 + sizeof(double) * nsys);
    ws.w_in_smem = (n * sizeof(double2) <= AR_SMEM_CAP);
    // partial sums of the whole-GPU Gram-Schmidt (forms other than the reference's)
    const int gsc = ref_dotc ? 0 : (int)((n + GS_ROWS - 1) / GS_ROWS);
    size_t oG = gsc ? carve(sizeof(double2) * nsys * gsc * (m + 1)) : 0;
    size_t oGn = gsc ? carve(sizeof(double) * nsys * gsc) : 0;
    ws.memb().ensure(bytes);
    char* base = ws.memb().as<char>();
    bt.X = reinterpret_cast<double2*>(base + oX);
    bt.B = reinterpret_cast<double2*>(base + oB);
    bt.Q = reinterpret_cast<double2*>(base + oQ);
    bt.gs_chunks = gsc;
    bt.gs_part = gsc ? reinterpret_cast<double2*>(base + oG) : nullptr;
    bt.gs_norm = gsc ? reinterpret_cast<double*>(base + oGn) : nullptr;
    bt.W = reinterpret_cast<double2*>(base + oW);
    bt.part = reinterpret_cast<double2*>(base + oP);
    bt.tickets = reinterpret_cast<int*>(base + oT);
    bt.small = reinterpret_cast<double2*>(base + oS);
    bt.small_stride = small;
    bt.st = reinterpret_cast<GmState*>(base + oSt);
    ws.norm_part = reinterpret_cast<double*>(base + oN);
    ws.anorm = ws.norm_part + (size_t)nsys * 1024;
    BEM_CUDA(cudaMemsetAsync(bt.tickets, 0, sizeof(int) * nsys * rb, ctx.stream));
    if (ws.w_in_smem) arnoldi_allow_smem(ctx.device);
    if (ws.graph_exec) {
        cudaGraphExecDestroy(ws.graph_exec);
        ws.graph_exec = nullptr;
    }
}

// Same layout as gm_prepare, carved from caller-provided device memory instead
// of an allocation.  Returns the bytes the layout needs; when that exceeds
// `capacity` nothing is written and the workspace is left unset.
size_t gm_prepare_external(Context& ctx, GmWorkspace& ws, int nsys, int64_t n, int m, const void* A, int64_t lda,
                           size_t mat_stride, bool fp32, bool ref_dotc, void* mem, size_t capacity) {
    const int64_t n_pad = (n + MV_ROWS - 1) / MV_ROWS * MV_ROWS;
    const size_t qstride = (size_t)n * (m + 1);
    const int rb = (int)((n + MV_ROWS - 1) / MV_ROWS), cb = (int)((n + MV_COLS - 1) / MV_COLS);
    const size_t small = gm_small_size(m);
    size_t bytes = 0;
    auto carve = [&](size_t b) { size_t o = bytes; bytes += (b + 255) / 256 * 256; return o; };
    size_t oX = carve(sizeof(double2) * nsys * n), oB = carve(sizeof(double2) * nsys * n);
    size_t oQ = carve(sizeof(double2) * nsys * qstride), oW = carve(sizeof(double2) * nsys * n);
    size_t oP = carve(sizeof(double2) * nsys * cb * n_pad), oT = carve(sizeof(int) * nsys * rb);
    size_t oS = carve(sizeof(double2) * nsys * small), oSt = carve(sizeof(GmState) * nsys);
    size_t oN = carve(sizeof(double) * nsys * 1024 + sizeof(double) * nsys);
    if (bytes > capacity) return bytes;
    GmBatch& bt = ws.bt;
    bt.nsys = nsys;
    bt.n = n;
    bt.n_pad = n_pad;
    bt.m = m;
    bt.A = A;
    bt.lda = lda;
    bt.mat_stride = mat_stride;
    bt.ref_dotc = ref_dotc ? 1 : 0;
    bt.qstride = qstride;
    ws.fp32 = fp32;
    ws.rb = rb;
    ws.cb = cb;
    bt.rb = rb;
    bt.cb = cb;
    bt.sys = nullptr;
    bt.ntiles = 0;
    ws.sys_host.clear();
    char* base = static_cast<char*>(mem);
    bt.X = reinterpret_cast<double2*>(base + oX);
    bt.B = reinterpret_cast<double2*>(base + oB);
    bt.Q = reinterpret_cast<double2*>(base + oQ);
    bt.gs_part = nullptr;  // caller memory: the single-CTA Gram-Schmidt
    bt.gs_norm = nullptr;
    bt.gs_chunks = 0;
    bt.W = reinterpret_cast<double2*>(base + oW);
    bt.part = reinterpret_cast<double2*>(base + oP);
    bt.tickets = reinterpret_cast<int*>(base + oT);
    bt.small = reinterpret_cast<double2*>(base + oS);
    bt.small_stride = small;
    bt.st = reinterpret_cast<GmState*>(base + oSt);
    ws.norm_part = reinterpret_cast<double*>(base + oN);
    ws.anorm = ws.norm_part + (size_t)nsys * 1024;
    // the last-CTA tickets must start at zero; every other region is written
    // before it is read
    BEM_CUDA(cudaMemsetAsync(bt.tickets, 0, sizeof(int) * nsys * rb, ctx.stream));
    ws.w_in_smem = (n * sizeof(double2) <= AR_SMEM_CAP);
    if (ws.w_in_smem) arnoldi_allow_smem(ctx.device);
    return bytes;
}

void gm_prepare_ragged(Context& ctx, GmWorkspace& ws, const std::vector<int64_t>& ns,
                       const std::vector<int64_t>& ldas, const std::vector<size_t>& a_offs, int m, const void* A,
                       bool fp32) {
    const int nsys = (int)ns.size();
    require(nsys >= 1 && ldas.size() == ns.size() && a_offs.size() == ns.size(), "ragged batch: bad layout");
    std::vector<GmSys>& sys = ws.sys_host;
    sys.assign(nsys, GmSys{});
    size_t v = 0, q = 0, p = 0, t = 0;
    int64_t tiles = 0, nmax = 0, npmax = 0;
    for (int s = 0; s < nsys; ++s) {
        GmSys& d = sys[s];
        d.n = ns[s];
        require(d.n >= 1 && ldas[s] >= d.n, "ragged batch: bad system size");
        d.lda = ldas[s];
        d.rb = (int)((d.n + MV_ROWS - 1) / MV_ROWS);
        d.cb = (int)((d.n + MV_COLS - 1) / MV_COLS);
        d.n_pad = (int64_t)d.rb * MV_ROWS;
        d.a_off = a_offs[s];
        d.v_off = v;
        d.q_off = q;
        d.p_off = p;
        d.t_off = t;
        d.tile0 = tiles;
        v += (size_t)d.n;
        q += (size_t)d.n * (m + 1);
        p += (size_t)d.cb * d.n_pad;
        t += (size_t)d.rb;
        tiles += (int64_t)d.rb * d.cb;
        nmax = std::max(nmax, d.n);
        npmax = std::max(npmax, d.n_pad);
    }
    GmBatch& bt = ws.bt;
    bt.nsys = nsys;
    bt.n = nmax;
    bt.n_pad = npmax;
    bt.m = m;
    bt.A = A;
    bt.lda = 0;
    bt.mat_stride = 0;
    bt.ref_dotc = 0;
    bt.qstride = 0;
    bt.rb = bt.cb = 0;
    bt.ntiles = tiles;
    ws.fp32 = fp32;
    ws.rb = ws.cb = 0;
    const size_t small = gm_small_size(m);
    size_t bytes = 0;
    auto carve = [&](size_t b) { size_t o = bytes; bytes += (b + 255) / 256 * 256; return o; };
    size_t oX = carve(sizeof(double2) * v), oB = carve(sizeof(double2) * v);
    size_t oQ = carve(sizeof(double2) * q), oW = carve(sizeof(double2) * v);
    size_t oP = carve(sizeof(double2) * p), oT = carve(sizeof(int) * t);
    size_t oS = carve(sizeof(double2) * nsys * small), oSt = carve(sizeof(GmState) * nsys);
    size_t oN = carve(sizeof(double) * nsys * 1024 + sizeof(double) * nsys);
    size_t oD = carve(sizeof(GmSys) * nsys);
    ws.w_in_smem = (nmax * sizeof(double2) <= AR_SMEM_CAP);
    // partial sums of the whole-GPU Gram-Schmidt
    const int gsc = (int)((nmax + GS_ROWS - 1) / GS_ROWS);
    size_t oG = carve(sizeof(double2) * nsys * gsc * (m + 1));
    size_t oGn = carve(sizeof(double) * nsys * gsc);
    ws.memb().ensure(bytes);
    char* base = ws.memb().as<char>();
    bt.X = reinterpret_cast<double2*>(base + oX);
    bt.B = reinterpret_cast<double2*>(base + oB);
    bt.Q = reinterpret_cast<double2*>(base + oQ);
    bt.gs_chunks = gsc;
    bt.gs_part = reinterpret_cast<double2*>(base + oG);
    bt.gs_norm = reinterpret_cast<double*>(base + oGn);
    bt.W = reinterpret_cast<double2*>(base + oW);
    bt.part = reinterpret_cast<double2*>(base + oP);
    bt.tickets = reinterpret_cast<int*>(base + oT);
    bt.small = reinterpret_cast<double2*>(base + oS);
    bt.small_stride = small;
    bt.st = reinterpret_cast<GmState*>(base + oSt);
    ws.norm_part = reinterpret_cast<double*>(base + oN);
    ws.anorm = ws.norm_part + (size_t)nsys * 1024;
    GmSys* dsys = reinterpret_cast<GmSys*>(base + oD);
    BEM_CUDA(cudaMemcpyAsync(dsys, sys.data(), sizeof(GmSys) * nsys, cudaMemcpyHostToDevice, ctx.stream));
    bt.sys = dsys;
    BEM_CUDA(cudaMemsetAsync(bt.tickets, 0, sizeof(int) * t, ctx.stream));
    if (ws.w_in_smem) arnoldi_allow_smem(ctx.device);
    if (ws.graph_exec) {
        cudaGraphExecDestroy(ws.graph_exec);
        ws.graph_exec = nullptr;
    }
}

size_t gm_q_total(const GmWorkspace& ws) {
    if (ws.sys_host.empty()) return (size_t)ws.bt.nsys * ws.bt.qstride;
    const GmSys& d = ws.sys_host.back();
    return d.q_off + (size_t)d.n * (ws.bt.m + 1);
}

void gm_matrix_norms(Context& ctx, GmWorkspace& ws) {
    const int nb = 512;
    if (!ws.sys_host.empty()) {
        for (int s = 0; s < ws.bt.nsys; ++s) {
            const GmSys& d = ws.sys_host[s];
            dim3 g1(nb, 1);
            if (ws.fp32)
                batch_frob_kernel<float2><<<g1, 256, 0, ctx.stream>>>(
                    static_cast<const float2*>(ws.bt.A) + d.a_off, d.n, d.lda, 0, ws.norm_part + (size_t)s * nb, nb);
            else
                batch_frob_kernel<double2><<<g1, 256, 0, ctx.stream>>>(
                    static_cast<const double2*>(ws.bt.A) + d.a_off, d.n, d.lda, 0, ws.norm_part + (size_t)s * nb,
                    nb);
            BEM_CHECK_LAUNCH(&ctx);
        }
        finish_norms_kernel<<<(ws.bt.nsys + 127) / 128, 128, 0, ctx.stream>>>(ws.norm_part, nb, ws.bt.nsys,
                                                                               ws.anorm);
        BEM_CHECK_LAUNCH(&ctx);
        return;
    }
    dim3 grid(nb, ws.bt.nsys);
    if (ws.fp32)
        batch_frob_kernel<float2><<<grid, 256, 0, ctx.stream>>>(ws.bt.A, ws.bt.n, ws.bt.lda, ws.bt.mat_stride,
                                                                ws.norm_part, nb);
    else
        batch_frob_kernel<double2><<<grid, 256, 0, ctx.stream>>>(ws.bt.A, ws.bt.n, ws.bt.lda, ws.bt.mat_stride,
                                                                 ws.norm_part, nb);
    BEM_CHECK_LAUNCH(&ctx);
    finish_norms_kernel<<<(ws.bt.nsys + 127) / 128, 128, 0, ctx.stream>>>(ws.norm_part, nb, ws.bt.nsys, ws.anorm);
    BEM_CHECK_LAUNCH(&ctx);
}

void gm_init(Context& ctx, GmWorkspace& ws, double tol, int64_t max_restarts) {
    gm_init_kernel<<<ws.bt.nsys, AR_THREADS, 0, ctx.stream>>>(ws.bt, ws.anorm, tol, max_restarts, nullptr, nullptr,
                                                              nullptr);
    BEM_CHECK_LAUNCH(&ctx);
}

void gm_init_each(Context& ctx, GmWorkspace& ws, const std::vector<double>& tol,
                  const std::vector<int64_t>& max_restarts, const std::vector<int>& m) {
    const size_t ns = (size_t)ws.bt.nsys;
    require(tol.size() == ns && max_restarts.size() == ns && m.size() == ns, "gmres: per-system settings");
    for (int x : m) require(x >= 1 && x <= ws.bt.m, "gmres: restart length above the batch's");
    ws.init_args.ensure(ns * (sizeof(double) + sizeof(int64_t) + sizeof(int)));
    char* base = ws.init_args.as<char>();
    BEM_CUDA(cudaMemcpyAsync(base, tol.data(), ns * sizeof(double), cudaMemcpyHostToDevice, ctx.stream));
    BEM_CUDA(cudaMemcpyAsync(base + ns * 8, max_restarts.data(), ns * sizeof(int64_t), cudaMemcpyHostToDevice,
                             ctx.stream));
    BEM_CUDA(cudaMemcpyAsync(base + ns * 16, m.data(), ns * sizeof(int), cudaMemcpyHostToDevice, ctx.stream));
    gm_init_kernel<<<ws.bt.nsys, AR_THREADS, 0, ctx.stream>>>(
        ws.bt, ws.anorm, 0.0, 0, reinterpret_cast<const double*>(base), reinterpret_cast<const int64_t*>(base + ns * 8),
        reinterpret_cast<const int*>(base + ns * 16));
    BEM_CHECK_LAUNCH(&ctx);
    ctx.sync();  // the host arrays are pageable and owned by the caller
}

static void launch_apply(Context& ctx, GmWorkspace& ws, int mode) {
    if (ws.hook) {
        ws.hook(ctx, ws, mode, ws.hook_user);
        return;
    }
    dim3 grid = ws.bt.sys ? dim3((unsigned)ws.bt.ntiles) : dim3((unsigned)ws.rb, (unsigned)ws.cb, (unsigned)ws.bt.nsys);
    if (ws.bt.split_lo) {
        gm_apply_kernel<float2, 2, 4><<<grid, MV_THREADS, 0, ctx.stream>>>(ws.bt, mode);
    } else if (ws.fp32) {
        if (mode == MV_Q) {
            // columns per load batch (loads in flight per thread), tuned per size
            const int u = ctx.tuning.pick("gm_apply_fp32", "unroll", ws.bt.n, ws.bt.nsys, MV_UNROLL);
            if (u == 4) gm_apply_kernel<float2, 0, 4><<<grid, MV_THREADS, 0, ctx.stream>>>(ws.bt, mode);
            else if (u == 16) gm_apply_kernel<float2, 0, 16><<<grid, MV_THREADS, 0, ctx.stream>>>(ws.bt, mode);
            else gm_apply_kernel<float2, 0, 8><<<grid, MV_THREADS, 0, ctx.stream>>>(ws.bt, mode);
        } else {
            gm_apply_kernel<float2, 1><<<grid, MV_THREADS, 0, ctx.stream>>>(ws.bt, mode);
        }
    } else {
        gm_apply_kernel<double2, 1><<<grid, MV_THREADS, 0, ctx.stream>>>(ws.bt, mode);
    }
    BEM_CHECK_LAUNCH(&ctx);
}

void gm_launch_iteration(Context& ctx, GmWorkspace& ws, cudaEvent_t ev_q0, cudaEvent_t ev_q1) {
    int nsys = ws.bt.nsys;
    launch_apply(ctx, ws, MV_START);
    gm_start_kernel<<<nsys, AR_THREADS, 0, ctx.stream>>>(ws.bt);
    BEM_CHECK_LAUNCH(&ctx);
    if (ws.precond) {
        if (ws.ev_p0) BEM_CUDA(cudaEventRecord(ws.ev_p0, ctx.stream));
        ws.precond(ctx, ws, MV_Q, ws.precond_user);
        if (ws.ev_p1) BEM_CUDA(cudaEventRecord(ws.ev_p1, ctx.stream));
    }
    if (ev_q0) BEM_CUDA(cudaEventRecord(ev_q0, ctx.stream));
    launch_apply(ctx, ws, MV_Q);
    if (ev_q1) BEM_CUDA(cudaEventRecord(ev_q1, ctx.stream));
    const bool gs = ws.bt.gs_part && !ws.bt.ref_dotc;
    if (gs) {
        const dim3 grid((unsigned)ws.bt.gs_chunks, (unsigned)nsys);
        const size_t hsm = sizeof(double2) * (size_t)(ws.bt.m + 1);
        for (int pass = 0; pass < 2; ++pass) {
            gm_gs_dots_kernel<<<grid, GS_THREADS, 0, ctx.stream>>>(ws.bt);
            BEM_CHECK_LAUNCH(&ctx);
            gm_gs_update_kernel<<<grid, GS_THREADS, hsm, ctx.stream>>>(ws.bt, pass);
            BEM_CHECK_LAUNCH(&ctx);
        }
    }
    size_t dyn = (!gs && ws.w_in_smem) ? (size_t)ws.bt.n * sizeof(double2) : 0;
    gm_arnoldi_kernel<<<nsys, AR_THREADS, dyn, ctx.stream>>>(ws.bt, (!gs && ws.w_in_smem) ? 1 : 0);
    BEM_CHECK_LAUNCH(&ctx);
    launch_apply(ctx, ws, MV_CHECK);
    gm_check_kernel<<<nsys, AR_THREADS, 0, ctx.stream>>>(ws.bt);
    BEM_CHECK_LAUNCH(&ctx);
}

void gm_read_states(Context& ctx, GmWorkspace& ws, std::vector<GmState>& out) {
    out.resize(ws.bt.nsys);
    BEM_CUDA(cudaMemcpyAsync(out.data(), ws.bt.st, sizeof(GmState) * ws.bt.nsys, cudaMemcpyDeviceToHost, ctx.stream));
    ctx.sync();
}

// The solve graph's loop test, run on the device after every round of
// `chunk` iterations: another round while some system is not done and the
// round cap is not reached (no host round trip between rounds).
__global__ void gm_continue_kernel(const GmState* __restrict__ st, int nsys, int* __restrict__ rounds, int max_rounds,
                                   cudaGraphConditionalHandle handle) {
    __shared__ int open;
    if (threadIdx.x == 0) open = 0;
    __syncthreads();
    for (int s = threadIdx.x; s < nsys; s += blockDim.x)
        if (!st[s].done) open = 1;
    __syncthreads();
    if (threadIdx.x == 0) {
        const int r = *rounds + 1;
        *rounds = r;
        cudaGraphSetConditional(handle, (open && r < max_rounds) ? 1u : 0u);
    }
}

// The whole solve as one graph: a conditional WHILE node whose body is
// `chunk` captured iterations plus the loop test.  Returns false (and leaves
// no error pending) where the runtime cannot build it.
static bool gm_build_solve_graph(Context& ctx, GmWorkspace& ws, int chunk, int max_rounds) {
    cudaGraph_t g = nullptr;
    if (cudaGraphCreate(&g, 0) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    cudaGraphConditionalHandle h;
    cudaGraphNodeParams np = {};
    cudaGraphNode_t node;
    bool ok = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault) == cudaSuccess;
    if (ok) {
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = h;
        np.conditional.type = cudaGraphCondTypeWhile;
        np.conditional.size = 1;
        ok = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np) == cudaSuccess;
    }
    if (ok) {
        cudaGraph_t body = np.conditional.phGraph_out[0];
        ok = cudaStreamBeginCaptureToGraph(ctx.stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) ==
             cudaSuccess;
        if (ok) {
            const int64_t before = ctx.launches;
            try {
                for (int c = 0; c < chunk; ++c) gm_launch_iteration(ctx, ws, nullptr, nullptr);
                gm_continue_kernel<<<1, 256, 0, ctx.stream>>>(ws.bt.st, ws.bt.nsys, ws.rounds.as<int>(), max_rounds,
                                                              h);
                BEM_CHECK_LAUNCH(&ctx);
            } catch (...) {
                cudaStreamEndCapture(ctx.stream, &body);  // leave the stream out of capture mode
                cudaGraphDestroy(g);
                ctx.launches = before;
                throw;
            }
            ws.launches_per_graph = ctx.launches - before;
            ctx.launches = before;
            ok = cudaStreamEndCapture(ctx.stream, &body) == cudaSuccess;
        }
    }
    if (ok) ok = cudaGraphInstantiate(&ws.graph_exec, g, 0) == cudaSuccess;
    cudaGraphDestroy(g);
    if (!ok) {
        cudaGetLastError();
        ws.graph_exec = nullptr;
    }
    return ok;
}

// Run to completion.  chunk == 0: one iteration at a time with a state read
// after each; chunk > 0: the solve graph (device-side loop over rounds of
// `chunk` iterations, one launch and one state read per solve), or where the
// runtime lacks conditional graph nodes a graph of `chunk` iterations with a
// state read after each launch.
void gm_run(Context& ctx, GmWorkspace& ws, int chunk, int64_t max_total_iterations) {
    std::vector<GmState> st, prev;
    int64_t issued = 0;
    if (chunk <= 0) {
        // one iteration at a time; with profiling, time the Krylov mat-vec of
        // every iteration with events on the launching stream
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        if (ctx.profiling) {
            BEM_CUDA(cudaEventCreate(&e0));
            BEM_CUDA(cudaEventCreate(&e1));
            if (ws.precond) {
                BEM_CUDA(cudaEventCreate(&ws.ev_p0));
                BEM_CUDA(cudaEventCreate(&ws.ev_p1));
            }
        }
        gm_read_states(ctx, ws, prev);
        for (;;) {
            gm_launch_iteration(ctx, ws, e0, e1);
            ++issued;
            gm_read_states(ctx, ws, st);
            if (ctx.profiling) {
                float ms = 0;
                BEM_CUDA(cudaEventElapsedTime(&ms, e0, e1));
                double entries = 0, mvs = 0;
                for (size_t s = 0; s < st.size(); ++s) {
                    const double ns = ws.sys_host.empty() ? (double)ws.bt.n : (double)ws.sys_host[s].n;
                    entries += (double)(st[s].iterations - prev[s].iterations) * ns * ns;
                    mvs += (double)(st[s].iterations - prev[s].iterations);
                }
                if (entries > 0)
                    ctx.stage_add(ws.mv_stage ? ws.mv_stage : (ws.fp32 ? "gmres_matvec_fp32" : "gmres_matvec_fp64"), ms,
                                  1, ws.mv_bytes > 0 ? ws.mv_bytes * mvs : entries * (ws.fp32 ? 8.0 : 16.0));
                if (ws.ev_p0 && entries > 0) {
                    float pms = 0;
                    BEM_CUDA(cudaEventElapsedTime(&pms, ws.ev_p0, ws.ev_p1));
                    ctx.stage_add("precond_apply", pms, 1, 0);
                }
            }
            prev = st;
            bool all = true;
            for (auto& s : st) all = all && s.done;
            if (all || issued >= max_total_iterations) break;
        }
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        if (ws.ev_p0) cudaEventDestroy(ws.ev_p0);
        if (ws.ev_p1) cudaEventDestroy(ws.ev_p1);
        ws.ev_p0 = ws.ev_p1 = nullptr;
        return;
    }
    const int max_rounds = (int)std::min<int64_t>((max_total_iterations + chunk - 1) / chunk, 1 << 30);
    if (!ws.graph_exec || ws.graph_chunk != chunk || ws.graph_rounds != max_rounds) {
        if (ws.graph_exec) cudaGraphExecDestroy(ws.graph_exec);
        ws.graph_exec = nullptr;
        ws.rounds.ensure(sizeof(int));
        ws.graph_loop = gm_build_solve_graph(ctx, ws, chunk, max_rounds);
        ws.graph_chunk = chunk;
        ws.graph_rounds = max_rounds;
    }
    if (ws.graph_loop) {
        int rounds = 0;
        BEM_CUDA(cudaMemsetAsync(ws.rounds.p, 0, sizeof(int), ctx.stream));
        BEM_CUDA(cudaGraphLaunch(ws.graph_exec, ctx.stream));
        BEM_CUDA(cudaMemcpyAsync(&rounds, ws.rounds.p, sizeof(int), cudaMemcpyDeviceToHost, ctx.stream));
        ctx.sync();
        ctx.launches += ws.launches_per_graph * rounds;
        return;
    }
    if (!ws.graph_exec) {
        cudaGraph_t g;
        int64_t before = ctx.launches;
        BEM_CUDA(cudaStreamBeginCapture(ctx.stream, cudaStreamCaptureModeThreadLocal));
        for (int c = 0; c < chunk; ++c) gm_launch_iteration(ctx, ws, nullptr, nullptr);
        BEM_CUDA(cudaStreamEndCapture(ctx.stream, &g));
        ws.launches_per_graph = ctx.launches - before;
        ctx.launches = before;
        BEM_CUDA(cudaGraphInstantiate(&ws.graph_exec, g, 0));
        cudaGraphDestroy(g);
        ws.graph_chunk = chunk;
    }
    for (;;) {
        BEM_CUDA(cudaGraphLaunch(ws.graph_exec, ctx.stream));
        ctx.launches += ws.launches_per_graph;
        issued += chunk;
        gm_read_states(ctx, ws, st);
        bool all = true;
        for (auto& s : st) all = all && s.done;
        if (all || issued >= max_total_iterations) break;
    }
}

// gmres.rs:35-59 GMRES::solve over one dense FP64 matrix on the device.
GmresResult gmres_dense_fp64(Context& ctx, int64_t n, const double2* A, int64_t lda, int64_t max_it, double tol,
                             double2* x) {
    if (max_it <= 0) max_it = 1000;
    if (max_it > n) max_it = n;
    if (tol <= 0.0) tol = 1e-5;
    int m = (int)std::ceil(std::sqrt((double)max_it));
    int64_t restarts = max_it / m;
    GmWorkspace ws;
    gm_prepare(ctx, ws, 1, n, m, A, lda, 0, false, true);
    BEM_CUDA(cudaMemcpyAsync(ws.bt.B, x, sizeof(double2) * n, cudaMemcpyDeviceToDevice, ctx.stream));
    gm_matrix_norms(ctx, ws);
    gm_init(ctx, ws, tol, restarts);
    gm_run(ctx, ws, 0, restarts * (int64_t)m + 1);
    std::vector<GmState> st;
    gm_read_states(ctx, ws, st);
    BEM_CUDA(cudaMemcpyAsync(x, ws.bt.X, sizeof(double2) * n, cudaMemcpyDeviceToDevice, ctx.stream));
    ctx.sync();
    GmresResult r;
    r.num_mv = st[0].num_mv;
    r.restarts = st[0].restarts + (st[0].converged ? 1 : 0);
    r.iterations = st[0].iterations;
    r.error = st[0].error;
    r.flag = st[0].converged ? 1 : 2;
    return r;
}

}  // namespace bem
