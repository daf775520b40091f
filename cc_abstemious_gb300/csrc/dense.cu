// Dense complex linear algebra for the plain FP64 form: partial-pivot LU
// (solve.rs:166-171 -> nalgebra lu()/solve_mut), triangular solves, GEMV and
// Frobenius norms.  All matrices column-major complex FP64 (double2).
#include "common.cuh"
#include "complex.cuh"

namespace bem {

constexpr int LU_NB = 32;

// ---------------------------------------------------------------------------
// Partial-pivot LU in panels of LU_NB columns.  Within a panel the columns are
// eliminated one launch each: the launch for column c scales column c below
// the diagonal and updates the rest of the panel, and its last CTA to finish
// picks column c + 1's pivot and swaps the two rows inside the panel.  The
// other columns take the panel's row swaps together afterwards
// (lu_laswp_kernel: nalgebra swaps whole rows at every step, and swaps of
// distinct columns commute), then the row block U12 and the trailing update.

// Pivot search (nalgebra icamax): first row r >= c maximising |re| + |im| of
// column c, by the whole CTA (a multiple of 32 threads, at most 1024); records
// piv[c] (and info on a zero column) and returns the row to every thread.
// Loads bypass L1: in the panel kernel the column was just written by other
// CTAs.
__device__ __forceinline__ int64_t lu_pivot_block(int64_t n, const double2* __restrict__ A, int64_t lda, int64_t c,
                                                  int32_t* __restrict__ piv, int* __restrict__ info) {
    __shared__ double bv[32];
    __shared__ int64_t bi[32];
    __shared__ int64_t res;
    const double2* col = A + c * lda;
    // four interleaved partial maxima keep four loads in flight
    double best = -1.0;
    int64_t bidx = c;
    const int64_t stride = blockDim.x;
    for (int64_t r0 = c + threadIdx.x; r0 < n; r0 += 4 * stride) {
        double v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int64_t r = r0 + u * stride;
            const double2 e = r < n ? __ldcg(col + r) : make_double2(-1.0, 0.0);
            v[u] = r < n ? fabs(e.x) + fabs(e.y) : -1.0;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (v[u] > best) {  // rows visited in increasing order per thread: first maximum kept
                best = v[u];
                bidx = r0 + u * stride;
            }
    }
    // warp and block reduction (ties -> smaller row index)
    for (int off = 16; off > 0; off >>= 1) {
        double ov = __shfl_down_sync(0xffffffffu, best, off);
        int64_t oi = __shfl_down_sync(0xffffffffu, bidx, off);
        if (ov > best || (ov == best && oi < bidx)) { best = ov; bidx = oi; }
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) { bv[w] = best; bi[w] = bidx; }
    __syncthreads();
    if (w == 0) {
        const int nw = blockDim.x >> 5;
        best = l < nw ? bv[l] : -1.0;
        bidx = l < nw ? bi[l] : c;
        for (int off = 16; off > 0; off >>= 1) {
            double ov = __shfl_down_sync(0xffffffffu, best, off);
            int64_t oi = __shfl_down_sync(0xffffffffu, bidx, off);
            if (ov > best || (ov == best && oi < bidx)) { best = ov; bidx = oi; }
        }
        if (l == 0) {
            piv[c] = (int32_t)bidx;
            if (best == 0.0 && *info == 0) *info = (int)(c + 1);
            res = bidx;
        }
    }
    __syncthreads();
    return res;
}

// Rows c and p swapped in the panel's columns [p0, pend).
__device__ __forceinline__ void lu_swap_panel(double2* __restrict__ A, int64_t lda, int64_t c, int64_t p, int64_t p0,
                                              int64_t pend) {
    if (p == c) return;
    for (int64_t j = p0 + threadIdx.x; j < pend; j += blockDim.x) {
        const double2 t = __ldcg(A + j * lda + c);
        A[j * lda + c] = __ldcg(A + j * lda + p);
        A[j * lda + p] = t;
    }
}

// The panel's first column: pivot and swap inside the panel.
__global__ void lu_pivot_swap_kernel(int64_t n, double2* __restrict__ A, int64_t lda, int64_t c, int64_t p0,
                                     int64_t pend, int32_t* __restrict__ piv, int* __restrict__ info) {
    const int64_t p = lu_pivot_block(n, A, lda, c, piv, info);
    lu_swap_panel(A, lda, c, p, p0, pend);
}

// gauss_step restricted to the panel: scale column c below the diagonal by
// 1/A[c,c] and apply the rank-1 update to panel columns c+1 .. pend-1 (one row
// per thread); then the last CTA pivots column c + 1 and swaps inside the
// panel.  `ticket` is zero on entry and left zero.
constexpr int LU_STEP_THREADS = 1024;
__global__ void __launch_bounds__(LU_STEP_THREADS) lu_panel_step_kernel(int64_t n, double2* __restrict__ A,
                                                                        int64_t lda, int64_t c, int64_t p0,
                                                                        int64_t pend, int32_t* __restrict__ piv,
                                                                        int* __restrict__ info,
                                                                        int* __restrict__ ticket) {
    __shared__ int last;
    const int64_t r = c + 1 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const double2 d = A[c * lda + c];
    if (r < n && !(d.x == 0.0 && d.y == 0.0)) {  // singular column: nalgebra skips the step
        const double2 inv = cdiv(make_double2(1.0, 0.0), d);
        const double2 l = cmul(A[c * lda + r], inv);
        A[c * lda + r] = l;
        for (int64_t j = c + 1; j < pend; ++j) {
            const double2 u = A[j * lda + c];
            double2 a = A[j * lda + r];
            cfma(a, cneg(l), u);
            A[j * lda + r] = a;
        }
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        last = atomicAdd(ticket, 1) == (int)gridDim.x - 1;
        if (last) *ticket = 0;
    }
    __syncthreads();
    if (!last || c + 1 >= pend) return;
    __threadfence();
    const int64_t p = lu_pivot_block(n, A, lda, c + 1, piv, info);
    lu_swap_panel(A, lda, c + 1, p, p0, pend);
}

// The panel's row swaps piv[p0 .. pend) applied in order to every column
// outside the panel (one thread per column).
__global__ void lu_laswp_kernel(int64_t n, double2* __restrict__ A, int64_t lda, int64_t p0, int64_t pend,
                                const int32_t* __restrict__ piv) {
    int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= n - (pend - p0)) return;
    if (j >= p0) j += pend - p0;
    double2* col = A + j * lda;
    for (int64_t c = p0; c < pend; ++c) {
        const int64_t p = piv[c];
        if (p == c) continue;
        const double2 t = col[c];
        col[c] = col[p];
        col[p] = t;
    }
}

// U12 = L11^{-1} A12 (unit lower nb x nb), one thread per column of A12.
__global__ void lu_trsm_kernel(double2* __restrict__ A, int64_t lda, int64_t p0, int nb, int64_t j0, int64_t ncols) {
    __shared__ double2 L[LU_NB][LU_NB + 1];
    for (int t = threadIdx.x; t < nb * nb; t += blockDim.x) {
        int r = t % nb, q = t / nb;
        L[r][q] = A[(p0 + q) * lda + p0 + r];
    }
    __syncthreads();
    int64_t j = j0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= j0 + ncols) return;
    double2 x[LU_NB];
    double2* col = A + j * lda + p0;
#pragma unroll
    for (int r = 0; r < LU_NB; ++r)
        if (r < nb) x[r] = col[r];
#pragma unroll
    for (int r = 0; r < LU_NB; ++r) {
        if (r >= nb) break;
        double2 v = x[r];
#pragma unroll
        for (int q = 0; q < LU_NB; ++q)
            if (q < r) cfma(v, cneg(L[r][q]), x[q]);
        x[r] = v;
        col[r] = v;
    }
}

// C -= A * B with A m x k (k <= LU_NB), B k x ncols, all sub-blocks of one
// column-major matrix.  64 x 64 output tile per CTA, 4 x 4 per thread, k
// staged through shared memory in slices of GK.
constexpr int GT = 64;
constexpr int GK = 16;
__global__ void __launch_bounds__(256) lu_gemm_kernel(double2* __restrict__ M, int64_t lda, int64_t r0, int64_t c0,
                                                      int64_t k0, int kk, int64_t m, int64_t ncols) {
    __shared__ double2 As[GK][GT + 1];
    __shared__ double2 Bs[GK][GT + 1];
    int64_t bi = r0 + (int64_t)blockIdx.x * GT;
    int64_t bj = c0 + (int64_t)blockIdx.y * GT;
    int tr = threadIdx.x % 16, tc = threadIdx.x / 16;
    double2 acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = make_double2(0, 0);
    for (int q0 = 0; q0 < kk; q0 += GK) {
        __syncthreads();
        for (int t = threadIdx.x; t < GT * GK; t += 256) {
            int r = t % GT, q = t / GT;
            As[q][r] = (q0 + q < kk && bi + r < r0 + m) ? M[(k0 + q0 + q) * lda + bi + r] : make_double2(0, 0);
            int q2 = t % GK, c = t / GK;
            Bs[q2][c] = (q0 + q2 < kk && bj + c < c0 + ncols) ? M[(bj + c) * lda + k0 + q0 + q2] : make_double2(0, 0);
        }
        __syncthreads();
        for (int q = 0; q < GK; ++q) {
            double2 av[4], bv[4];
#pragma unroll
            for (int a = 0; a < 4; ++a) av[a] = As[q][tr + 16 * a];
#pragma unroll
            for (int b = 0; b < 4; ++b) bv[b] = Bs[q][tc + 16 * b];
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) cfma(acc[a][b], av[a], bv[b]);
        }
    }
#pragma unroll
    for (int b = 0; b < 4; ++b) {
        int64_t j = bj + tc + 16 * b;
        if (j >= c0 + ncols) continue;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            int64_t i = bi + tr + 16 * a;
            if (i >= r0 + m) continue;
            double2 v = M[j * lda + i];
            v.x -= acc[a][b].x;
            v.y -= acc[a][b].y;
            M[j * lda + i] = v;
        }
    }
}

void lu_factor_fp64(Context& ctx, int64_t n, double2* A, int64_t lda, int32_t* d_piv, int* d_info) {
    BEM_CUDA(cudaMemsetAsync(d_info, 0, sizeof(int), ctx.stream));
    ctx.w_flags.ensure(256);
    int* ticket = ctx.w_flags.as<int>() + 2;  // [0] device error, [1] the caller's info
    BEM_CUDA(cudaMemsetAsync(ticket, 0, sizeof(int), ctx.stream));
    for (int64_t p0 = 0; p0 < n; p0 += LU_NB) {
        int nb = (int)std::min<int64_t>(LU_NB, n - p0);
        int64_t pend = p0 + nb;
        lu_pivot_swap_kernel<<<1, 1024, 0, ctx.stream>>>(n, A, lda, p0, p0, pend, d_piv, d_info);
        BEM_CHECK_LAUNCH(&ctx);
        for (int64_t c = p0; c < pend && c + 1 < n; ++c) {
            const int64_t rows = n - c - 1;
            lu_panel_step_kernel<<<(unsigned)((rows + LU_STEP_THREADS - 1) / LU_STEP_THREADS), LU_STEP_THREADS, 0,
                                   ctx.stream>>>(n, A, lda, c, p0, pend, d_piv, d_info, ticket);
            BEM_CHECK_LAUNCH(&ctx);
        }
        if (n > nb) {
            lu_laswp_kernel<<<(unsigned)((n - nb + 255) / 256), 256, 0, ctx.stream>>>(n, A, lda, p0, pend, d_piv);
            BEM_CHECK_LAUNCH(&ctx);
        }
        int64_t rest = n - pend;
        if (rest <= 0) continue;
        lu_trsm_kernel<<<(unsigned)((rest + 127) / 128), 128, 0, ctx.stream>>>(A, lda, p0, nb, pend, rest);
        BEM_CHECK_LAUNCH(&ctx);
        dim3 grid((unsigned)((rest + GT - 1) / GT), (unsigned)((rest + GT - 1) / GT));
        lu_gemm_kernel<<<grid, 256, 0, ctx.stream>>>(A, lda, pend, pend, p0, nb, rest, rest);
        BEM_CHECK_LAUNCH(&ctx);
    }
}

// ---------------------------------------------------------------------------
// Triangular solves with the packed LU, blocked by LU_NB: the diagonal block
// is solved by one CTA, the rest of the vector updated by a GEMV.
__global__ void apply_pivots_kernel(int64_t n, const int32_t* __restrict__ piv, double2* __restrict__ b) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    for (int64_t c = 0; c < n; ++c) {
        int64_t p = piv[c];
        if (p != c) {
            double2 t = b[c];
            b[c] = b[p];
            b[p] = t;
        }
    }
}

// lower == 1: unit lower forward substitution on rows [p0, p0+nb);
// lower == 0: upper backward substitution.
__global__ void trsv_block_kernel(const double2* __restrict__ A, int64_t lda, int64_t p0, int nb, int lower,
                                  double2* __restrict__ b, int* __restrict__ info) {
    if (threadIdx.x != 0) return;
    if (lower) {
        for (int r = 0; r < nb; ++r) {
            double2 v = b[p0 + r];
            for (int q = 0; q < r; ++q) cfma(v, cneg(A[(p0 + q) * lda + p0 + r]), b[p0 + q]);
            b[p0 + r] = v;
        }
    } else {
        for (int r = nb - 1; r >= 0; --r) {
            double2 v = b[p0 + r];
            for (int q = r + 1; q < nb; ++q) cfma(v, cneg(A[(p0 + q) * lda + p0 + r]), b[p0 + q]);
            double2 d = A[(p0 + r) * lda + p0 + r];
            if (d.x == 0.0 && d.y == 0.0) { if (*info == 0) *info = (int)(p0 + r + 1); v = make_double2(0, 0); }
            else v = cdiv(v, d);
            b[p0 + r] = v;
        }
    }
}

// b[rows] -= A[rows, p0:p0+nb] * b[p0:p0+nb]
__global__ void trsv_update_kernel(const double2* __restrict__ A, int64_t lda, int64_t r0, int64_t m, int64_t p0,
                                   int nb, double2* __restrict__ b) {
    __shared__ double2 xs[LU_NB];
    if (threadIdx.x < nb) xs[threadIdx.x] = b[p0 + threadIdx.x];
    __syncthreads();
    int64_t i = r0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= r0 + m) return;
    double2 v = b[i];
    for (int q = 0; q < nb; ++q) cfma(v, cneg(A[(p0 + q) * lda + i]), xs[q]);
    b[i] = v;
}

void lu_solve_fp64(Context& ctx, int64_t n, const double2* A, int64_t lda, const int32_t* d_piv, double2* b) {
    int* info = ctx.w_flags.as<int>() + 1;
    apply_pivots_kernel<<<1, 32, 0, ctx.stream>>>(n, d_piv, b);
    BEM_CHECK_LAUNCH(&ctx);
    for (int64_t p0 = 0; p0 < n; p0 += LU_NB) {
        int nb = (int)std::min<int64_t>(LU_NB, n - p0);
        trsv_block_kernel<<<1, 32, 0, ctx.stream>>>(A, lda, p0, nb, 1, b, info);
        BEM_CHECK_LAUNCH(&ctx);
        int64_t m = n - p0 - nb;
        if (m > 0) {
            trsv_update_kernel<<<(unsigned)((m + 255) / 256), 256, 0, ctx.stream>>>(A, lda, p0 + nb, m, p0, nb, b);
            BEM_CHECK_LAUNCH(&ctx);
        }
    }
    int64_t last = ((n - 1) / LU_NB) * LU_NB;
    for (int64_t p0 = last; p0 >= 0; p0 -= LU_NB) {
        int nb = (int)std::min<int64_t>(LU_NB, n - p0);
        trsv_block_kernel<<<1, 32, 0, ctx.stream>>>(A, lda, p0, nb, 0, b, info);
        BEM_CHECK_LAUNCH(&ctx);
        if (p0 > 0) {
            trsv_update_kernel<<<(unsigned)((p0 + 255) / 256), 256, 0, ctx.stream>>>(A, lda, 0, p0, p0, nb, b);
            BEM_CHECK_LAUNCH(&ctx);
        }
    }
}

// ---------------------------------------------------------------------------
// y = alpha A x + beta y (m x n).  Column chunks are reduced by the last CTA of
// each row block in a fixed order (deterministic).
constexpr int GV_ROWS = 256;
constexpr int GV_COLS = 256;
__global__ void __launch_bounds__(GV_ROWS) gemv64_kernel(int64_t m, int64_t n, const double2* __restrict__ A,
                                                         int64_t lda, const double2* __restrict__ x,
                                                         double2* __restrict__ y, z2 alpha, z2 beta,
                                                         double2* __restrict__ part, int* __restrict__ tickets) {
    __shared__ double2 xs[GV_COLS];
    __shared__ int last;
    int64_t i = blockIdx.x * (int64_t)GV_ROWS + threadIdx.x;
    int64_t j0 = (int64_t)blockIdx.y * GV_COLS;
    int64_t jn = min((int64_t)GV_COLS, n - j0);
    for (int t = threadIdx.x; t < jn; t += GV_ROWS) xs[t] = x[j0 + t];
    __syncthreads();
    double2 acc = make_double2(0, 0);
    if (i < m) {
        const double2* a = A + j0 * lda + i;
        int64_t q = 0;
        for (; q + 4 <= jn; q += 4) {
            double2 a0 = a[q * lda], a1 = a[(q + 1) * lda], a2 = a[(q + 2) * lda], a3 = a[(q + 3) * lda];
            cfma(acc, a0, xs[q]);
            cfma(acc, a1, xs[q + 1]);
            cfma(acc, a2, xs[q + 2]);
            cfma(acc, a3, xs[q + 3]);
        }
        for (; q < jn; ++q) cfma(acc, a[q * lda], xs[q]);
        part[(int64_t)blockIdx.y * m + i] = acc;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = (atomicAdd(&tickets[blockIdx.x], 1) == (int)gridDim.y - 1);
    __syncthreads();
    if (!last) return;
    __threadfence();
    if (i < m) {
        double2 s = make_double2(0, 0);
        for (int c = 0; c < (int)gridDim.y; ++c) s = cadd(s, part[(int64_t)c * m + i]);
        double2 v = cmul(alpha, s);
        if (beta.x != 0.0 || beta.y != 0.0) cfma(v, beta, y[i]);
        y[i] = v;
    }
    if (threadIdx.x == 0) tickets[blockIdx.x] = 0;  // reset for the next launch
}

void gemv_fp64(Context& ctx, int64_t m, int64_t n, const double2* A, int64_t lda, const double2* x, double2* y,
               cd alpha, cd beta) {
    unsigned rb = (unsigned)((m + GV_ROWS - 1) / GV_ROWS), cb = (unsigned)((n + GV_COLS - 1) / GV_COLS);
    ctx.w_small.ensure(sizeof(double2) * (size_t)cb * m + 4096 * sizeof(int));
    // tickets live after the partials; zeroed once and reset by the kernel
    static_assert(sizeof(int) == 4, "");
    double2* part = ctx.w_small.as<double2>();
    int* tickets = reinterpret_cast<int*>(part + (size_t)cb * m);
    require(rb <= 4096, "gemv: too many row blocks");
    BEM_CUDA(cudaMemsetAsync(tickets, 0, sizeof(int) * rb, ctx.stream));
    dim3 grid(rb, cb);
    gemv64_kernel<<<grid, GV_ROWS, 0, ctx.stream>>>(m, n, A, lda, x, y, make_double2(alpha.re, alpha.im),
                                                    make_double2(beta.re, beta.im), part, tickets);
    BEM_CHECK_LAUNCH(&ctx);
}

// ---------------------------------------------------------------------------
__global__ void frob64_kernel(int64_t m, int64_t n, const double2* __restrict__ A, int64_t lda,
                              double* __restrict__ part) {
    __shared__ double red[256];
    double s = 0;
    int64_t total = m * n;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        int64_t j = t / m, i = t - j * m;
        double2 v = A[j * lda + i];
        s += v.x * v.x + v.y * v.y;
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

double frob_norm_fp64(Context& ctx, int64_t m, int64_t n, const double2* A, int64_t lda) {
    const int nb = 1024;
    DevBuf d;
    d.ensure(sizeof(double) * nb);
    frob64_kernel<<<nb, 256, 0, ctx.stream>>>(m, n, A, lda, d.as<double>());
    BEM_CHECK_LAUNCH(&ctx);
    std::vector<double> h(nb);
    BEM_CUDA(cudaMemcpyAsync(h.data(), d.p, sizeof(double) * nb, cudaMemcpyDeviceToHost, ctx.stream));
    ctx.sync();
    double s = 0;
    for (double v : h) s += v;
    return std::sqrt(s);
}

}  // namespace bem
