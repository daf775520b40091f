// Mixed-precision LU preconditioner for the batched GMRES.
//
// Every operator of the batch (FP32 complex, column-major) is copied and
// factored A = L U without pivoting, in blocks of LB = 128 unknowns, all
// systems of a (possibly ragged) batch advancing block step k together, the
// trailing updates delayed over groups of G steps (4 or 8, by size):
//
//   diag   one CTA per system: L11^-1 and U11^-1 of the diagonal block in one
//          register-tiled elimination sweep (tiny pivots are replaced and
//          counted); the two inverses are kept per block (strict lower /
//          upper of one tile) and written in the real embedding below for
//          the panel GEMMs.
//   l21    the column panel A21 is embedded (memory-bound copy), then
//          L21 = A21 U11^-1 on the tensor cores, in place (the embedding is a
//          ring homomorphism: emb(A U) = emb(A) emb(U)); the GEMM's epilogue
//          also writes L21 in natural form into the factors.
//   u12    U12 = L11^-1 A12 on the tensor cores into a side buffer (the
//          trailing update's second operand), copied into the factors after.
//   gemm   A22 -= L21 U12 on the tensor cores (tcgen05, kind::f16 with FP16
//          operands, FP32 accumulation in tensor memory).  FP16 keeps TF32's
//          11-bit significand at half the operand bytes and twice the MMA
//          rate; the panel GEMMs write FP16 copies of L21 (clamped to the FP16
//          range) and of U12 scaled by a power of two per system (2^10 over
//          the operator's largest entry, undone in the epilogue), so the
//          entries that matter stay normal numbers.  The complex product is one real
//          GEMM: with A' the 2m x 2k real matrix holding [[ar, -ai], [ai, ar]]
//          per complex entry, A' times the natural real view of U12
//          (2k x n, re/im interleaved along the rows, which is how the
//          column-major complex storage reads as floats) gives the natural
//          real view of the product.  Tiles of 128 real rows x 256 columns,
//          K = 256 per step of the group in chunks of 32 (up to 1024: the
//          group's panels side by side) staged by 2-D tensor copies (TMA) in the
//          128-byte swizzled K-major layout; a persistent warp-specialised kernel
//          (producer warp, MMA warp, eight epilogue warps, a four-stage operand
//          ring and two tensor-memory accumulators) so that operand loads, MMAs
//          and the read-modify-write of A22 overlap; every wait is bounded.
//
// Applying M = U^-1 L^-1 to a Krylov vector (flexible right preconditioning:
// Z[:, k] = M Q[:, k]) is a blocked forward and back substitution with the
// kept diagonal-block inverses in one launch (row tickets, flags), FP32
// factors and arithmetic (the Krylov vectors stay FP64).  The factorization is TF32-accurate, which is plenty for a
// preconditioner: the FP64 outer GMRES with exact residuals decides the
// answer, the factors only decide the iteration count.
#include <cuda.h>
#include <cuda_fp16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <memory>

#include "common.cuh"
#include "complex.cuh"
#include "gmres.cuh"
#include "kernels.cuh"
#include "precond.cuh"
#include "umma.cuh"

namespace bem {

namespace {

constexpr int LB = 128;                 // block size (complex unknowns)
constexpr int GM = 128, GN = 256;       // GEMM tile: real rows x columns
constexpr int GK = 32;                  // real K per pipeline chunk (FP32 operands, panel GEMMs)
constexpr int GCHUNKS = 2 * LB / GK;    // 8 chunks: K = 256, one block step
constexpr int GK16 = 64;                // real K per pipeline chunk (FP16 operands, trailing update)
constexpr int GCHUNKS16 = 2 * LB / GK16;  // 4 chunks: K = 256, one block step
// Block steps per delayed trailing update (a factorization's group size G):
// the panel workspace is WK = 2 LB G wide (K = 256 G per pass over A22).
// Eight steps halve the A22 traffic per flop of four at twice the workspace
// and longer in-group updates, which pay off for large systems only.
constexpr int LU_GROUP_MAX = 8;
}  // namespace
// smallest system size for which eight-step groups are allowed (the memory
// budgets of the batched forms reserve their workspace from this size on)
constexpr int64_t LU_GROUP8_MIN_N = 4096;
namespace {
constexpr int GS = 4;                   // pipeline stages
constexpr int GTHREADS = 320;           // producer warp, MMA warp, eight epilogue warps
constexpr int GEPI = GTHREADS - 64;     // epilogue threads
constexpr uint32_t GA_BYTES = GM * GK * 4, GB_BYTES = GN * GK * 4, GSTAGE = GA_BYTES + GB_BYTES;
constexpr uint32_t G_SMEM = GS * GSTAGE + 256;  // stages + barriers + tensor-memory slot + abort flag
constexpr uint32_t G_TMEM_COLS = 512;           // two accumulators of GN columns

struct LuSys {
    float2* F;    // factors (copy of the operator), column-major, leading dimension ld
    float2* Dm;   // per block: L11^-1 (strict lower) and U11^-1 (upper), LB x LB column-major
    float* W;     // real embedding of the current step's column panel A21: 2n rows x 2 LB floats
    float* Li;    // real embedding of L11^-1: 2 LB x 2 LB, row-major
    float* UiT;   // transposed real embedding of U11^-1: 2 LB x 2 LB, row-major
    float* Y;     // the group's U12, natural real view: column j at Y + WK j (step k + j at rows 256 j ..)
    const CUtensorMap* tmW;  // W: 2n rows x 2 LB floats, 128-byte swizzled 32 x 128 boxes
    const CUtensorMap* tmF;  // F's natural real view: n columns x 2n floats, 32 x 256 boxes
    const CUtensorMap* tmY;  // Y: n columns x WK floats, 32 x 256 boxes
    const CUtensorMap* tmL;  // Li: 256 rows, 32 x 128 boxes
    const CUtensorMap* tmU;  // UiT: 256 rows, 32 x 256 boxes
    __half* W16;  // W after the L21 GEMM in FP16 (the trailing update's A operand)
    __half* Y16;  // ysc Y in FP16 (its B operand)
    const CUtensorMap* tmW16;  // W16: 2n rows x WK halves, 64 x 128 boxes
    const CUtensorMap* tmY16;  // Y16: n columns x WK halves, 64 x 256 boxes
    float ysc, yinv;  // power-of-two scale of Y16 and its inverse
    int64_t n, ld;
    int nblk, wk;     // blocks; panel workspace width 2 LB G
};

// One entry per (system, launch): the system, its first CTA in the flattened
// grid of that launch and, for the GEMMs, the region it covers (rows of the
// panel workspace, relative to the step group's trailing origin, and columns).
struct LuWork {
    int sys, tiles_i;
    int64_t tile0;
    int64_t r0, r1, c0, c1;
};

// Index of the work entry holding CTA t of a launch, and t's rank in it.
__device__ __forceinline__ int lu_entry(const LuWork* __restrict__ wl, int nw, int64_t t, int64_t& local) {
    int lo = 0, hi = nw - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (wl[mid].tile0 <= t) lo = mid;
        else hi = mid - 1;
    }
    local = t - wl[lo].tile0;
    return lo;
}

__device__ __forceinline__ int lu_locate(const LuWork* __restrict__ wl, int nw, int64_t t, int64_t& local) {
    int lo = 0, hi = nw - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (wl[mid].tile0 <= t) lo = mid;
        else hi = mid - 1;
    }
    local = t - wl[lo].tile0;
    return wl[lo].sys;
}

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ void cfmaf_(float2& acc, float2 a, float2 b) {
    acc.x = fmaf(a.x, b.x, fmaf(-a.y, b.y, acc.x));
    acc.y = fmaf(a.x, b.y, fmaf(a.y, b.x, acc.y));
}

// FP32 rounding of an FP64 operator buffer.
__global__ void lu_round_kernel(const double2* __restrict__ A, size_t n, float2* __restrict__ F) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double2 v = A[i];
        F[i] = make_float2((float)v.x, (float)v.y);
    }
}

// ---------------------------------------------------------------------------
// Diagonal block: LU without pivoting and both triangular inverses in one
// elimination sweep.  Z starts as the block; at step j, with pivot p = Z[j][j],
// column c_i = Z[i][j] and row r_c = Z[j][c]:
//   Z[i][c] -= c_i r_c / p   for i != j, c != j, and (i > j or c > j)
//   Z[i][j]  = -c_i / p (i > j),  c_i / p (i < j);   Z[j][c] = -r_c / p (c > j)
//   Z[j][j]  = 1 / p
// Entries with i > j and c > j follow the Schur complement, so c_i / p = L[i][j]
// and r_c = U[j][c]; the strictly lower part then collects L^-1 by row
// operations and the upper part U^-1 by column operations (the region i < j,
// c < j is final).  On exit Z = L^-1 (strictly lower, unit diagonal implied)
// + U^-1 (upper): the two inverses the triangular solves and panels use.
// DIAG_THREADS threads (DW warps), each holding a 4 x DB tile of Z in
// registers (rows tx + 32a, columns ty + DW b); one barrier per step.  The
// steps run in groups of DW columns, so the tile column (b = j / DW) and row
// (a = j / 32) of step j are compile-time constants: the owners' stores take
// no register indexing, and the final region i < j, c < j is skipped by whole
// tile blocks.
constexpr int DIAG_THREADS = 512;
constexpr int DIAG_TS = LB + 1;  // column stride of the block in shared memory
constexpr int DW = DIAG_THREADS / 32, DB = LB / DW;  // warps (column stride), columns per thread
static_assert(32 % DW == 0 || DW % 32 == 0, "a group of DW columns lies in one 32-row tile block");

template <int JB>
__device__ __forceinline__ void lu_diag_group(float2 (&z)[4][DB], int nb, int tx, int ty, float2 (*colbuf)[LB],
                                              float2 (*rowbuf)[LB], int* __restrict__ small_pivots) {
    constexpr int JA = DW * JB / 32;
#pragma unroll 1
    for (int jc = 0; jc < DW; ++jc) {
        const int j = DW * JB + jc, jl = j & 31;
        if (j >= nb) return;
        float2* cb = colbuf[j & 1];
        float2* rb = rowbuf[j & 1];
        if (ty == jc)
#pragma unroll
            for (int a = 0; a < 4; ++a) cb[tx + 32 * a] = z[a][JB];
        if (tx == jl)
#pragma unroll
            for (int b = 0; b < DB; ++b) rb[ty + DW * b] = z[JA][b];
        __syncthreads();  // (double-buffered: the next step writes the other pair)
        float2 p = rb[j];
        float pn = p.x * p.x + p.y * p.y;
        const bool tiny = !(pn > 1e-30f);  // also catches NaN
        if (tiny) {
            p = make_float2(1e-15f, 0.f);
            pn = 1e-30f;
            if (threadIdx.x == 0) atomicAdd(small_pivots, 1);
        }
        const float rn = __frcp_rn(pn);  // one reciprocal for both parts
        const float2 pinv = make_float2(p.x * rn, -p.y * rn);
        // row multipliers c_i / p; row j takes 1 + 1/p, which turns its
        // entries right of the pivot into -r_c / p through the same update
        const bool below = tx > jl;  // row tx + 32 JA is below row j
        float2 cvs[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            cvs[a] = cmulf(cb[tx + 32 * a], pinv);
            if (a == JA && tx == jl) cvs[a] = make_float2(1.f + pinv.x, pinv.y);
        }
        const float2 cvb = below ? cvs[JA] : make_float2(0.f, 0.f);  // row JA, columns left of j
#pragma unroll
        for (int b = 0; b < DB; ++b) {
            float2 r = rb[ty + DW * b];
            if (b == JB) {
                const float2 hi = ty > jc ? r : make_float2(0.f, 0.f);  // columns right of j only
                if (ty == jc) r = make_float2(0.f, 0.f);
#pragma unroll
                for (int a = 0; a < 4; ++a) {
                    const float2 v = a < JA ? hi : (a > JA ? r : (below ? r : hi));
                    cfmaf_(z[a][b], make_float2(-cvs[a].x, -cvs[a].y), v);
                }
            } else {
#pragma unroll
                for (int a = 0; a < 4; ++a) {
                    if (b < JB && a < JA) continue;  // final region
                    const float2 m = (b < JB && a == JA) ? cvb : cvs[a];
                    cfmaf_(z[a][b], make_float2(-m.x, -m.y), r);
                }
            }
        }
        if (ty == jc)  // column j: -L[i][j] below, U^-1 entries above, 1/p on the diagonal
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                const int r = tx + 32 * a;
                z[a][JB] = r > j ? make_float2(-cvs[a].x, -cvs[a].y) : (r < j ? cvs[a] : pinv);
            }
    }
}

template <int JB>
__device__ __forceinline__ void lu_diag_sweep(float2 (&z)[4][DB], int nb, int tx, int ty, float2 (*colbuf)[LB],
                                              float2 (*rowbuf)[LB], int* __restrict__ small_pivots) {
    if constexpr (JB < LB / DW) {
        lu_diag_group<JB>(z, nb, tx, ty, colbuf, rowbuf, small_pivots);
        lu_diag_sweep<JB + 1>(z, nb, tx, ty, colbuf, rowbuf, small_pivots);
    }
}

__global__ void __launch_bounds__(DIAG_THREADS) lu_diag_kernel(const LuSys* __restrict__ sys,
                                                               const LuWork* __restrict__ wl, int k,
                                                               int* __restrict__ small_pivots) {
    // LB x LB, column-major with a padded column stride: T[c * DIAG_TS + r]
    // (reads along a row then fall in distinct banks)
    extern __shared__ float2 T[];
    __shared__ float2 colbuf[2][LB], rowbuf[2][LB];
    const LuSys S = sys[wl[blockIdx.x].sys];
    const int64_t k0 = (int64_t)k * LB;
    const int nb = (int)min((int64_t)LB, S.n - k0);
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    float2 z[4][DB];
#pragma unroll
    for (int b = 0; b < DB; ++b) {
        const int c = ty + DW * b;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const int r = tx + 32 * a;
            // outside the block: identity, untouched by the sweep over j < nb
            z[a][b] = (r < nb && c < nb) ? S.F[(k0 + c) * S.ld + k0 + r] : make_float2(r == c ? 1.f : 0.f, 0.f);
        }
    }
    lu_diag_sweep<0>(z, nb, tx, ty, colbuf, rowbuf, small_pivots);
#pragma unroll
    for (int b = 0; b < DB; ++b)
#pragma unroll
        for (int a = 0; a < 4; ++a) T[(ty + DW * b) * DIAG_TS + tx + 32 * a] = z[a][b];
    __syncthreads();
    float2* Dk = S.Dm + (size_t)k * LB * LB;
    for (int c = ty; c < nb; c += DIAG_THREADS / 32)
        for (int r = tx; r < nb; r += 32) Dk[c * LB + r] = T[c * DIAG_TS + r];
    if (nb < LB || S.n <= k0 + LB) return;  // no panels after the last block
    // real embeddings for the panel GEMMs: Li = [[re, -im], [im, re]] of
    // L11^-1 (unit lower), UiT = the transpose of that of U11^-1 (upper)
    float2* Li2 = reinterpret_cast<float2*>(S.Li);
    float2* Ui2 = reinterpret_cast<float2*>(S.UiT);
    for (int t = threadIdx.x; t < LB * LB; t += blockDim.x) {
        const int i = t / LB, p = t % LB;  // Li: element (i, p), consecutive threads along a row of Li
        const float2 l = p < i ? T[p * DIAG_TS + i] : make_float2(p == i ? 1.f : 0.f, 0.f);
        Li2[(2 * i) * LB + p] = make_float2(l.x, -l.y);
        Li2[(2 * i + 1) * LB + p] = make_float2(l.y, l.x);
        const int pu = t % LB, q = t / LB;  // UiT rows 2q, 2q + 1 from U11^-1 (pu, q)
        const float2 u = pu <= q ? T[q * DIAG_TS + pu] : make_float2(0.f, 0.f);
        Ui2[(2 * q) * LB + pu] = make_float2(u.x, u.y);
        Ui2[(2 * q + 1) * LB + pu] = make_float2(-u.y, u.x);
    }
}

// W <- real embedding of step ks's column panel A21 (64 rows per CTA): rows
// 2(i - kt_w) and 2(i - kt_w) + 1 of W hold [ar, -ai] and [ai, ar] for every
// column of A21's row i; kt_w = (kw + 1) LB is the trailing origin of the
// step group.  (The L21 GEMM reads it once; the trailing updates read the
// FP16 copy of L21 the GEMM writes into W16 at column woff.)
__global__ void __launch_bounds__(256) lu_expand_kernel(const LuSys* __restrict__ sys, const LuWork* __restrict__ wl,
                                                        int nw, int ks, int kw) {
    extern __shared__ float2 Y[];  // 64 x LB, column stride 65: Y[p * 65 + i] (at most two-way bank conflicts)
    constexpr int NT = 256, PAIRS = 32 * LB / NT;  // row pairs per thread
    int64_t tile;
    const LuSys S = sys[lu_locate(wl, nw, blockIdx.x, tile)];
    const int64_t k0 = (int64_t)ks * LB, kt = k0 + LB, ktw = (int64_t)(kw + 1) * LB, i0 = kt + 64 * tile;
    const int nrow = (int)min((int64_t)64, S.n - i0);
    // rows i, i + 1 of column p in one 16-byte load, all of a thread's loads
    // in flight together.  Aligned: ld is even (the factors' tensor map has a
    // 16-byte column stride) and i0 + i is even.  In bounds: row i + 1 = n
    // only for odd n, where ld >= n + 1.
    float4 v[PAIRS];
#pragma unroll
    for (int q = 0; q < PAIRS; ++q) {
        const int t = threadIdx.x + NT * q, p = t / 32, i = 2 * (t % 32);
        v[q] = i < nrow ? *reinterpret_cast<const float4*>(S.F + (k0 + p) * S.ld + i0 + i)
                        : make_float4(0.f, 0.f, 0.f, 0.f);
    }
#pragma unroll
    for (int q = 0; q < PAIRS; ++q) {
        const int t = threadIdx.x + NT * q, p = t / 32, i = 2 * (t % 32);
        Y[p * 65 + i] = make_float2(v[q].x, v[q].y);
        Y[p * 65 + i + 1] = make_float2(v[q].z, v[q].w);
    }
    __syncthreads();
    // two columns per thread: 16-byte stores into both rows of the embedding
    const int64_t wr0 = 2 * (i0 - ktw);
    for (int t = threadIdx.x; t < nrow * (LB / 2); t += NT) {
        const int i = t / (LB / 2), c = 2 * (t % (LB / 2));
        const float2 a = Y[c * 65 + i], b = Y[(c + 1) * 65 + i];
        float4* w0 = reinterpret_cast<float4*>(S.W + (wr0 + 2 * i) * (2 * LB));
        float4* w1 = reinterpret_cast<float4*>(S.W + (wr0 + 2 * i + 1) * (2 * LB));
        w0[c / 2] = make_float4(a.x, -a.y, b.x, -b.y);
        w1[c / 2] = make_float4(a.y, a.x, b.y, b.x);
    }
}

// Step ks's row panel in the factors (rows ks LB .. + LB of every column
// j >= (ks + 1) LB) <- rows yoff .. yoff + 256 of Y (32 columns per CTA).
__global__ void __launch_bounds__(256) lu_copy_u12_kernel(const LuSys* __restrict__ sys,
                                                          const LuWork* __restrict__ wl, int nw, int ks, int yoff) {
    int64_t tile;
    const LuSys S = sys[lu_locate(wl, nw, blockIdx.x, tile)];
    const int64_t k0 = (int64_t)ks * LB, kt = k0 + LB, j0 = kt + 32 * tile;
    const int ncol = (int)min((int64_t)32, S.n - j0);
    for (int t = threadIdx.x; t < ncol * (LB / 2); t += blockDim.x) {
        const int c = t / (LB / 2), q = t % (LB / 2);  // 64 float4 per column
        const float4 v = reinterpret_cast<const float4*>(S.Y + (j0 + c) * S.wk + yoff)[q];
        reinterpret_cast<float4*>(S.F + (j0 + c) * S.ld + k0)[q] = v;
    }
}

// ---------------------------------------------------------------------------
// Trailing update on the tensor cores.

// 2-D tensor copy global -> shared (tensor map in global memory), completing
// on the mbarrier, with an L2 eviction policy (createpolicy): the GEMM operands
// are panels that every tile of a launch re-reads, so they are kept in L2
// (evict_last) while the trailing block streams past them.
__device__ __forceinline__ uint64_t l2_policy_evict_last() {
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}

__device__ __forceinline__ void tma_load_2d_hint(uint32_t dst, const CUtensorMap* tmap, int x, int y, uint64_t* bar,
                                                 uint64_t policy) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint"
        " [%0], [%1, {%2, %3}], [%4], %5;" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(tmap)), "r"(x), "r"(y), "r"(smem_u32(bar)), "l"(policy)
        : "memory");
}

// Shared-memory descriptor of a K-major operand in the 128-byte swizzle
// layout written by the tensor copies: rows of 128 bytes, 8-row atoms of
// 1024 bytes (stride between atoms), descriptor version bit 46, layout type 2.
// The start address moves 32 bytes per MMA along K inside the atom.
__device__ __forceinline__ uint64_t umma_desc_sw128(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)1 << 16;             // leading byte offset (unused for this layout)
    d |= (uint64_t)(1024 >> 4) << 32;   // stride byte offset
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;             // 128-byte swizzle
    return d;
}

__device__ __forceinline__ void umma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void umma_f16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// Instruction descriptor, kind::f16: FP16 A and B (format 0, both K-major), FP32 D.
__host__ __device__ constexpr uint32_t umma_idesc_f16_f32(int M, int N) {
    return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// Instruction descriptor, kind::tf32: TF32 A and B (both K-major), FP32 D.
__host__ __device__ constexpr uint32_t umma_idesc_tf32_f32(int M, int N) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// Persistent, warp-specialised trailing update.  One thread of warp 0 stages
// operand chunks with two tensor copies each into a ring of GS stages (the
// copies complete on the stage's "full" barrier), lane 0 of warp 1 issues
// the MMAs of a stage and releases it through tcgen05.commit on its "empty"
// barrier, and warps 2-9 drain the accumulator of the previous tile (two
// accumulators of 256 tensor-memory columns) while the next tile's MMAs run.
// GEMM modes (D = A' B over K = 32 nchunks real), for block step ks of the
// step group starting at kw (trailing origin kt_w = (kw + 1) LB, the row origin
// of W, W16 and of the TRAIL work regions):
//   TRAIL  A22 -= W16 Y16    128 rows of W16 x 256 columns of Y16 (FP16) inside
//                            each work entry's region; K = 256 per step of the
//                            group applied (up to 256 G for the rest of A22)
//   U12    Y = Li U12raw     the two 128-row halves of Li x 256 columns of the
//                            step's row panel, into Y's (and scaled into Y16's)
//                            rows yoff .. yoff + 256
//   L21    W16 = W UiT^T     128 rows of W x all 256 columns, into W16 at column
//                            woff; L21 in natural form into the factors
enum { G_TRAIL = 0, G_U12 = 1, G_L21 = 2 };

struct GemmTile {
    const CUtensorMap *tmA, *tmB;
    int ax, ay, bx, by;  // tensor-copy coordinates of chunk 0 (x advances by GK per chunk)
    float *F, *Y, *W;
    __half *Y16, *W16;
    float ysc, yinv;
    int64_t n, ld, ld2, k0, ktw, row0, rows_end, col0, col_end, wk;
};

// Raster of a TRAIL region's tiles (tiles_i row tiles x tiles_j column
// tiles): bands of sb_c column tiles, each swept by super-blocks of sb_r row
// tiles x the band's columns, row tiles fastest.  A band's slice of the row
// panel Y (sb_c x 1 MB at K = 1024) stays in L2 while the band's rows stream
// the column panel W past it, so W is read once per band and Y once per
// launch (column-after-column order re-reads W for every column tile, which
// for n >= 12000 is larger than L2).  (sb_r, sb_c) comes from the tuning
// table.
__device__ __forceinline__ void raster_tile(int64_t local, int64_t tiles_i, int64_t tiles_j, int sb_r, int sb_c,
                                            int64_t& ti, int64_t& tj) {
    const int64_t per_band = tiles_i * sb_c;
    const int64_t band = local / per_band, rem = local - band * per_band;
    const int64_t bc = min((int64_t)sb_c, tiles_j - band * sb_c);  // columns of this band
    const int64_t sr = rem / (sb_r * bc), rem2 = rem - sr * (sb_r * bc);
    const int64_t br = min((int64_t)sb_r, tiles_i - sr * sb_r);     // rows of this super-block
    ti = sr * sb_r + rem2 % br;
    tj = band * sb_c + rem2 / br;
}

template <int MODE>
__device__ __forceinline__ GemmTile gemm_tile(const LuSys* __restrict__ sys, const LuWork* __restrict__ wl, int nw,
                                              int64_t t, int ks, int kw, int woff, int raster) {
    int64_t local;
    const LuWork& w = wl[lu_entry(wl, nw, t, local)];
    const LuSys S = sys[w.sys];
    GemmTile g;
    g.F = reinterpret_cast<float*>(S.F);
    g.Y = S.Y;
    g.W = S.W;
    g.Y16 = S.Y16;
    g.W16 = S.W16;
    g.ysc = S.ysc;
    g.yinv = S.yinv;
    g.wk = S.wk;
    g.n = S.n;
    g.ld = S.ld;
    g.ld2 = 2 * S.ld;
    g.k0 = (int64_t)ks * LB;
    g.ktw = (int64_t)(kw + 1) * LB;
    if (MODE == G_TRAIL) {
        int64_t ti, tj;
        raster_tile(local, w.tiles_i, (w.c1 - w.c0 + GN - 1) / GN, raster >> 16, raster & 0xFFFF, ti, tj);
        g.row0 = w.r0 + ti * GM;
        g.rows_end = w.r1;
        g.col0 = w.c0 + tj * GN;
        g.col_end = w.c1;
        g.tmA = S.tmW16;
        g.ax = 0;
        g.ay = (int)g.row0;
        g.tmB = S.tmY16;
        g.bx = 0;
        g.by = (int)g.col0;
    } else if (MODE == G_U12) {
        g.row0 = (local & 1) * GM;
        g.rows_end = 2 * LB;
        g.col0 = w.c0 + (local >> 1) * GN;
        g.col_end = w.c1;
        g.tmA = S.tmL;
        g.ax = 0;
        g.ay = (int)g.row0;
        g.tmB = S.tmF;
        g.bx = (int)(2 * g.k0);
        g.by = (int)g.col0;
    } else {
        g.row0 = w.r0 + local * GM;
        g.rows_end = w.r1;
        g.col0 = 0;
        g.col_end = 2 * LB;
        g.tmA = S.tmW;
        g.ax = 0;
        g.ay = (int)g.row0;
        g.tmB = S.tmU;
        g.bx = 0;
        g.by = 0;
    }
    return g;
}

template <int MODE>
__global__ void __launch_bounds__(GTHREADS, 1) lu_gemm_kernel(const LuSys* __restrict__ sys,
                                                              const LuWork* __restrict__ wl, int nw, int ks, int kw,
                                                              int nchunks, int woff, int yoff, int64_t ntiles,
                                                              int raster,
                                                              int* __restrict__ err) {
    extern __shared__ __align__(1024) unsigned char smem[];
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + GS * GSTAGE);
    uint64_t* empty = full + GS;
    uint64_t* tfull = empty + GS;
    uint64_t* tempty = tfull + 2;
    uint64_t* drain = tempty + 2;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (warp == 0) tmem_alloc(tmem_slot, G_TMEM_COLS);
    if (tid == 0) {
        for (int s = 0; s < GS; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int a = 0; a < 2; ++a) {
            mbar_init(&tfull[a], 1);
            mbar_init(&tempty[a], GEPI);
        }
        mbar_init(drain, 1);
        *abort_flag = 0;
        fence_mbar_init();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t base = smem_u32(smem);
    auto fail = [&]() {
        *abort_flag = 1;
        atomicOr(err, DEVERR_MBAR_TIMEOUT);
    };

    if (warp == 0) {
        // ---- producer: one thread, two tensor copies per stage
        if (lane == 0) {
            const uint64_t keep = l2_policy_evict_last();
            int64_t it = 0;
            for (int64_t t = blockIdx.x; t < ntiles && !*abort_flag; t += gridDim.x) {
                const GemmTile g = gemm_tile<MODE>(sys, wl, nw, t, ks, kw, woff, raster);
                for (int c = 0; c < nchunks; ++c, ++it) {
                    const int st = (int)(it % GS);
                    const int64_t round = it / GS;
                    if (round > 0 && !mbar_wait_bounded(&empty[st], (uint32_t)((round - 1) & 1))) {
                        fail();
                        break;
                    }
                    const uint32_t As = base + st * GSTAGE, Bs = As + GA_BYTES;
                    mbar_arrive_expect_tx(&full[st], GSTAGE);
                    const int kx = c * (MODE == G_TRAIL ? GK16 : GK);  // 128 bytes per chunk row
                    tma_load_2d_hint(As, g.tmA, g.ax + kx, g.ay, &full[st], keep);
                    tma_load_2d_hint(Bs, g.tmB, g.bx + kx, g.by, &full[st], keep);
                }
            }
            if (*abort_flag) {
                // copies may still be landing in the last stages: wait for them
                for (int64_t j = it > GS ? it - GS : 0; j < it; ++j)
                    mbar_wait_bounded(&full[j % GS], (uint32_t)((j / GS) & 1));
            }
        }
        __syncwarp();
    } else if (warp == 1) {
        // ---- MMA issuer
        const uint32_t idesc = MODE == G_TRAIL ? umma_idesc_f16_f32(GM, GN) : umma_idesc_tf32_f32(GM, GN);
        int64_t it = 0, tc = 0;
        for (int64_t t = blockIdx.x; t < ntiles && !*abort_flag; t += gridDim.x, ++tc) {
            const int acc = (int)(tc & 1);
            const int64_t use = tc >> 1;
            if (lane == 0 && use > 0 && !mbar_wait_bounded(&tempty[acc], (uint32_t)((use - 1) & 1))) fail();
            __syncwarp();
            if (*abort_flag) break;
            tc_fence_after();
            for (int c = 0; c < nchunks; ++c, ++it) {
                const int st = (int)(it % GS);
                if (lane == 0) {
                    if (!mbar_wait_bounded(&full[st], (uint32_t)((it / GS) & 1))) fail();
                    else {
                        tc_fence_after();
                        const uint32_t a = base + st * GSTAGE, b = a + GA_BYTES;
                        // four MMAs per 128-byte chunk row: K = 8 (TF32) or 16 (FP16),
                        // 32 bytes of the row each
#pragma unroll
                        for (int kk = 0; kk < 4; ++kk) {
                            if (MODE == G_TRAIL)
                                umma_f16(tmem + (uint32_t)(acc * GN), umma_desc_sw128(a + kk * 32),
                                         umma_desc_sw128(b + kk * 32), idesc, (c | kk) ? 1u : 0u);
                            else
                                umma_tf32(tmem + (uint32_t)(acc * GN), umma_desc_sw128(a + kk * 32),
                                          umma_desc_sw128(b + kk * 32), idesc, (c | kk) ? 1u : 0u);
                        }
                        umma_commit(&empty[st]);
                    }
                }
                __syncwarp();
                if (*abort_flag) break;
            }
            if (*abort_flag) break;
            if (lane == 0) umma_commit(&tfull[acc]);
            __syncwarp();
        }
    } else {
        // ---- epilogue: A22 -= accumulator; two warps per lane quarter, each
        // with half of the columns
        const int quarter = warp & 3;  // tensor-memory lanes this warp may read
        const int half = (warp - 2) >> 2;
        const uint32_t lane_base = (uint32_t)(32 * quarter) << 16;
        int64_t tc = 0;
        for (int64_t t = blockIdx.x; t < ntiles && !*abort_flag; t += gridDim.x, ++tc) {
            const int acc = (int)(tc & 1);
            if (!mbar_wait_bounded(&tfull[acc], (uint32_t)((tc >> 1) & 1))) {
                fail();
                break;
            }
            tc_fence_after();
            const GemmTile g = gemm_tile<MODE>(sys, wl, nw, t, ks, kw, woff, raster);
            const int64_t r = g.row0 + 32 * quarter + lane;
            const bool rok = r < g.rows_end;
            for (int cc = half * (GN / 64); cc < (half + 1) * (GN / 64); ++cc) {
                const int64_t jb = g.col0 + cc * 32;
                if (jb >= g.col_end) break;  // uniform over the warp
                float v[32];
                tmem_ld32(tmem + lane_base + (uint32_t)(acc * GN + cc * 32), v);
                if (MODE == G_TRAIL) {
                    if (!rok) continue;
                    // all 32 loads in flight before the first store; the
                    // trailing block is touched once per launch: streaming
                    // (evict-first) loads and stores keep the panels in L2
                    const int nq = (int)min((int64_t)32, g.col_end - jb);
                    float* p0 = g.F + jb * g.ld2 + 2 * g.ktw + r;
                    float cv[32];
#pragma unroll
                    for (int q = 0; q < 32; ++q) cv[q] = q < nq ? __ldcs(p0 + q * g.ld2) : 0.f;
#pragma unroll
                    for (int q = 0; q < 32; ++q)
                        if (q < nq) __stcs(p0 + q * g.ld2, fmaf(-v[q], g.yinv, cv[q]));
                } else if (MODE == G_U12) {
                    const int nq = (int)min((int64_t)32, g.col_end - jb);
                    float* p0 = g.Y + jb * g.wk + yoff + r;
                    __half* h0 = g.Y16 + jb * g.wk + yoff + r;
#pragma unroll
                    for (int q = 0; q < 32; ++q)
                        if (q < nq) {
                            p0[q * g.wk] = v[q];
                            h0[q * g.wk] = __float2half_rn(fminf(fmaxf(v[q] * g.ysc, -65504.f), 65504.f));
                        }
                } else {
                    // L21: the embedded row in FP16 into W16 (the trailing
                    // updates' operand), and the natural entries into the
                    // factors (row 2i holds re, row 2i + 1 im of column 2p)
                    float im[16];
#pragma unroll
                    for (int q = 0; q < 16; ++q) im[q] = __shfl_down_sync(0xffffffffu, v[2 * q], 1);
                    if (!rok) continue;
                    uint4* hrow = reinterpret_cast<uint4*>(g.W16 + r * g.wk + woff + cc * 32);
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        uint32_t h[4];
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            const __half2 x = __floats2half2_rn(fminf(fmaxf(v[8 * q + 2 * e], -65504.f), 65504.f),
                                                                fminf(fmaxf(v[8 * q + 2 * e + 1], -65504.f), 65504.f));
                            h[e] = *reinterpret_cast<const uint32_t*>(&x);
                        }
                        hrow[q] = make_uint4(h[0], h[1], h[2], h[3]);
                    }
                    if ((lane & 1) == 0) {
                        const int64_t i = g.ktw + (r >> 1);
                        float2* F2 = reinterpret_cast<float2*>(g.F);
#pragma unroll
                        for (int q = 0; q < 16; ++q)
                            F2[(g.k0 + cc * 16 + q) * g.ld + i] = make_float2(v[2 * q], im[q]);
                    }
                }
            }
            tc_fence_before();
            mbar_arrive(&tempty[acc]);
        }
    }
    __syncthreads();
    if (*abort_flag) {
        // every MMA this CTA issued is tracked by one more commit
        if (tid == 32) umma_commit(drain);
        if (tid == 32) mbar_wait_bounded(drain, 0);
        __syncthreads();
    }
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tmem, G_TMEM_COLS);
}

// ---------------------------------------------------------------------------
// Preconditioner application z = U^-1 L^-1 q: both block substitutions in one
// launch.  A ticket is one block row of one system in one direction:
//   forward  row b:  y = q_b - sum_{k<b} L_bk z_k,    z_b = y + (L_bb^-1 - I) y
//   backward row b:  w = z_b - sum_{k>b} U_bk z_k,    z_b = U_bb^-1 w
// CTAs take tickets from a counter in an order where every row a ticket
// depends on has a smaller ticket (forward rows by b, then backward rows by
// descending b, systems interleaved), so a CTA only waits for rows that CTAs
// already running hold.  A finished row publishes its flag; a set flag also
// says every row it depended on is final, so a row polls only when it reaches
// blocks past the last flag it saw.  Waits are bounded (error flag, then the
// row carries on).  Block products run in FP32 (TF32-accurate factors),
// accumulated over blocks in FP64.
struct LuTicket {
    int sys, nrhs;   // systems sys .. sys + nrhs - 1 share one operator (several right-hand sides)
    int phase, row;  // 0 forward / 1 backward, block row
    int flags;       // the group's forward flags, then its backward flags
};

__device__ __forceinline__ int ld_acquire_gpu(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_gpu(int* p, int v) {
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Thread 0 waits (bounded) until flag f is set.
__device__ __forceinline__ void lu_wait_flag(const int* f, int* err) {
    for (uint32_t it = 0; it < (1u << 24); ++it) {
        if (ld_acquire_gpu(f)) return;
        __nanosleep(100);
    }
    atomicOr(err, DEVERR_BARRIER_TIMEOUT);
}

constexpr int TS_THREADS = 256;  // 64 row pairs x 4 column quarters of a block
constexpr int TS_MAXR = 4;       // right-hand sides per ticket (systems sharing one operator)

// Sixteen columns c0 .. c0 + 15 of a block B (columns at col, stride ld,
// float2 entries) for the row pair of this thread, one float4 per column
// (zero past the block's nc columns or below its rows).
__device__ __forceinline__ void lu_block_load(const float2* __restrict__ col, int64_t ld, int c0, int nc,
                                              bool rows_ok, float4 (&e)[16]) {
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const int c = c0 + i;
        e[i] = rows_ok && c < nc ? __ldg(reinterpret_cast<const float4*>(col + (int64_t)c * ld))
                                 : make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

// (a0, a1)[r] += those sixteen columns times v[r][c0 ..] for every right-hand
// side r < R (v in shared memory), in column order.
template <int R>
__device__ __forceinline__ void lu_block_fma(const float4 (&e)[16], const float2 (*v)[LB], int c0, float2 (&a0)[R],
                                             float2 (&a1)[R]) {
#pragma unroll
    for (int i = 0; i < 16; ++i)
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const float2 x = v[r][c0 + i];
            cfmaf_(a0[r], make_float2(e[i].x, e[i].y), x);
            cfmaf_(a1[r], make_float2(e[i].z, e[i].w), x);
        }
}

// R = the largest group of right-hand sides in the ticket list (1, 2 or 4):
// smaller groups leave their unused vectors at zero.
template <int R>
__global__ void __launch_bounds__(TS_THREADS, R == TS_MAXR ? 1 : 2) lu_trsv_kernel(const LuSys* __restrict__ sys,
                                                             const LuTicket* __restrict__ tickets, int ntickets,
                                                             int* __restrict__ counter, int* __restrict__ flags,
                                                             GmBatch bt, int* __restrict__ err) {
    __shared__ float2 xs[R][LB];
    __shared__ double2 red[4][LB];
    __shared__ double2 ys[R][LB];
    __shared__ int tk, all_final;
    const int rp = threadIdx.x & 63, cq = threadIdx.x >> 6;
    for (;;) {
        if (threadIdx.x == 0) tk = atomicAdd(counter, 1);
        __syncthreads();
        const int t = tk;
        __syncthreads();  // every thread has read tk
        if (t >= ntickets) return;
        const LuTicket T = tickets[t];
        // the group's vectors: inactive systems (converged, or at another
        // stage) keep zero vectors and are not written
        bool act[R];
        double2* zr[R];
        const double2* qr[R];
        bool any = false;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            act[r] = false;
            zr[r] = nullptr;
            qr[r] = nullptr;
            if (r < T.nrhs) {
                const GmState& st = bt.st[T.sys + r];
                act[r] = gm_apply_active(bt, st, MV_Q);
                const GmView g = gm_view(bt, T.sys + r);
                zr[r] = bt.Z + g.q + (size_t)st.k * g.n;
                qr[r] = bt.Q + g.q + (size_t)st.k * g.n;
                any = any || act[r];
            }
        }
        if (!any) continue;
        const LuSys S = sys[T.sys];
        const int b = T.row, nblk = S.nblk;
        const int nr = (int)min((int64_t)LB, S.n - (int64_t)b * LB);
        const bool rows_ok = 2 * rp < nr;  // nr is even or the block's last
        const bool fwd = T.phase == 0;
        int* fl = flags + T.flags + (fwd ? 0 : nblk);
        double2 acc[R][2];
#pragma unroll
        for (int r = 0; r < R; ++r) acc[r][0] = acc[r][1] = make_double2(0, 0);
        // blocks of the row, in the order their values become final
        const int nk = fwd ? b : nblk - 1 - b;
        int seen = 0;  // blocks known final
        if (!fwd && threadIdx.x == 0) lu_wait_flag(flags + T.flags + nblk - 1, err);  // forward done
        __syncthreads();
        for (int i = 0; i < nk; ++i) {
            const int k = fwd ? i : nblk - 1 - i;
            const int nc = (int)min((int64_t)LB, S.n - (int64_t)k * LB);
            const float2* col = S.F + (int64_t)k * LB * S.ld + (int64_t)b * LB + 2 * rp;
            // the factors are final: the first half of this thread's quarter of
            // the block is requested before the wait for z_k and its staging
            float4 e[16];
            lu_block_load(col, S.ld, 32 * cq, nc, rows_ok, e);
            if (i >= seen) {
                if (threadIdx.x == 0) {
                    // the row's last dependency first: once set, all are
                    const int ok = ld_acquire_gpu(fl + (fwd ? b - 1 : b + 1));
                    if (!ok) lu_wait_flag(fl + k, err);
                    all_final = ok;
                }
                __syncthreads();
                seen = all_final ? nk : i + 1;
            }
            for (int u = threadIdx.x; u < R * LB; u += TS_THREADS) {
                const int r = u / LB, c = u % LB;
                double2 v = make_double2(0, 0);
#pragma unroll
                for (int q = 0; q < R; ++q)
                    if (q == r && act[q] && c < nc) v = __ldcg(zr[q] + (int64_t)k * LB + c);
                xs[r][c] = make_float2((float)v.x, (float)v.y);
            }
            __syncthreads();
            // acc[r] += B v[r] over this thread's 32-column quarter, summed in
            // FP32 within the block
            float2 a0[R], a1[R];
#pragma unroll
            for (int r = 0; r < R; ++r) a0[r] = a1[r] = make_float2(0.f, 0.f);
            lu_block_fma<R>(e, xs, 32 * cq, a0, a1);
            lu_block_load(col, S.ld, 32 * cq + 16, nc, rows_ok, e);
            lu_block_fma<R>(e, xs, 32 * cq + 16, a0, a1);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                acc[r][0].x += a0[r].x;
                acc[r][0].y += a0[r].y;
                acc[r][1].x += a1[r].x;
                acc[r][1].y += a1[r].y;
            }
            __syncthreads();  // xs reused by the next block
        }
        // the diagonal block's first half is requested before the reductions
        const float2* D = S.Dm + (size_t)b * LB * LB + 2 * rp;
        float4 e[16];
        lu_block_load(D, LB, 32 * cq, nr, rows_ok, e);
        // y = source - sum, per right-hand side
#pragma unroll
        for (int r = 0; r < R; ++r) {
            red[cq][2 * rp] = acc[r][0];
            red[cq][2 * rp + 1] = acc[r][1];
            __syncthreads();
            if (threadIdx.x < LB) {
                const int i = threadIdx.x;
                double2 y = make_double2(0, 0);
                if (i < nr && act[r]) {
                    y = fwd ? qr[r][(int64_t)b * LB + i] : __ldcg(zr[r] + (int64_t)b * LB + i);
                    for (int q = 0; q < 4; ++q) {
                        y.x -= red[q][i].x;
                        y.y -= red[q][i].y;
                    }
                }
                ys[r][i] = y;
                xs[r][i] = make_float2((float)y.x, (float)y.y);
            }
            __syncthreads();
        }
        // diagonal block: strictly lower part of L_bb^-1 (unit diagonal
        // added in FP64) or the upper part of U_bb^-1 with its diagonal
        float2 d0[R], d1[R];
#pragma unroll
        for (int r = 0; r < R; ++r) d0[r] = d1[r] = make_float2(0.f, 0.f);
        {
            const int r0 = 2 * rp;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                if (h == 1) lu_block_load(D, LB, 32 * cq + 16, nr, rows_ok, e);
#pragma unroll
                for (int i = 0; i < 16; ++i) {
                    const int c = 32 * cq + 16 * h + i;
                    if (!rows_ok || c >= nr) continue;
                    const bool u0 = fwd ? c < r0 : c >= r0, u1 = fwd ? c < r0 + 1 : c >= r0 + 1;
#pragma unroll
                    for (int r = 0; r < R; ++r) {
                        const float2 x = xs[r][c];
                        if (u0) cfmaf_(d0[r], make_float2(e[i].x, e[i].y), x);
                        if (u1) cfmaf_(d1[r], make_float2(e[i].z, e[i].w), x);
                    }
                }
            }
        }
#pragma unroll
        for (int r = 0; r < R; ++r) {
            red[cq][2 * rp] = make_double2(d0[r].x, d0[r].y);
            red[cq][2 * rp + 1] = make_double2(d1[r].x, d1[r].y);
            __syncthreads();
            if (threadIdx.x < LB && threadIdx.x < nr && act[r]) {
                const int i = threadIdx.x;
                double2 v = fwd ? ys[r][i] : make_double2(0, 0);
                for (int q = 0; q < 4; ++q) {
                    v.x += red[q][i].x;
                    v.y += red[q][i].y;
                }
                __stcg(zr[r] + (int64_t)b * LB + i, v);
            }
            __syncthreads();
        }
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) st_release_gpu(fl + b, 1);
    }
}

// ---------------------------------------------------------------------------
struct LuData {
    DevBuf sysbuf, work, info, maps;
    std::vector<LuSys> sys;
    int nblk_max = 0;
    int group = 4;  // block steps per delayed trailing update
    // work lists: per launch, [offset, count, ctas] into `work`
    struct Seg {
        int64_t off = 0;
        int count = 0;
        int64_t ctas = 0;
    };
    // the factorization as an ordered list of launches
    enum Kind { DIAG, EXPAND, L21, U12, COPY, TRAIL };
    struct Launch {
        Kind kind;
        int ks, kw, woff, yoff, nchunks;
        Seg seg;
    };
    std::vector<Launch> plan;
    // preconditioner application: tickets, and a counter + row flags
    DevBuf tickets, flags;
    int ntickets = 0, nflags = 0, trsv_grid = 1, trsv_r = 1;  // trsv_r: right-hand sides per ticket
    std::vector<LuWork> host;
    int small_pivots = 0;
};

// A work entry: system, CTAs, and for the GEMMs the covered region.
struct Entry {
    int sys;
    int64_t ctas;
    int tiles_i;
    int64_t r0, r1, c0, c1;
};

LuData::Seg add_segment(LuData& d, const std::vector<Entry>& entries) {
    LuData::Seg sg;
    sg.off = (int64_t)d.host.size();
    int64_t t = 0;
    for (const Entry& e : entries) {
        if (e.ctas <= 0) continue;
        d.host.push_back(LuWork{e.sys, e.tiles_i, t, e.r0, e.r1, e.c0, e.c1});
        t += e.ctas;
    }
    sg.count = (int)((int64_t)d.host.size() - sg.off);
    sg.ctas = t;
    return sg;
}

// A GEMM region of TRAIL mode: rows [r0, r1) of W (relative to the trailing
// origin) x columns [c0, c1).
Entry trail_entry(int s, int64_t r0, int64_t r1, int64_t c0, int64_t c1) {
    const int64_t ti = (r1 - r0 + GM - 1) / GM, tj = (c1 - c0 + GN - 1) / GN;
    return Entry{s, (r1 > r0 && c1 > c0) ? ti * tj : 0, (int)ti, r0, r1, c0, c1};
}

void lu_hook(Context& c, GmWorkspace& ws, int mode, void* user) {
    (void)mode;
    LuData& d = *static_cast<LuData*>(user);
    if (!d.ntickets) return;
    BEM_CUDA(cudaMemsetAsync(d.flags.p, 0, sizeof(int) * (size_t)d.nflags, c.stream));
    int* f = d.flags.as<int>();
    const LuSys* sys = d.sysbuf.as<LuSys>();
    const LuTicket* tk = d.tickets.as<LuTicket>();
    if (d.trsv_r == 1)
        lu_trsv_kernel<1><<<(unsigned)d.trsv_grid, TS_THREADS, 0, c.stream>>>(sys, tk, d.ntickets, f, f, ws.bt,
                                                                              device_err(c));
    else if (d.trsv_r == 2)
        lu_trsv_kernel<2><<<(unsigned)d.trsv_grid, TS_THREADS, 0, c.stream>>>(sys, tk, d.ntickets, f, f, ws.bt,
                                                                              device_err(c));
    else
        lu_trsv_kernel<TS_MAXR><<<(unsigned)d.trsv_grid, TS_THREADS, 0, c.stream>>>(sys, tk, d.ntickets, f, f,
                                                                                    ws.bt, device_err(c));
    BEM_CHECK_LAUNCH(&c);
}

}  // namespace

// The driver's tensor-map encoder, looked up through the runtime (the library
// then needs no link-time dependency on the driver library).
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        BEM_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q));
        require(p != nullptr && q == cudaDriverEntryPointSuccess, "cuTensorMapEncodeTiled unavailable", BEM_ERR_CUDA);
        fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

int lu_group(const Context& c, int64_t nmin, int64_t nsys) {
    // eight steps only where every factored system is large: the workspace
    // doubles and the in-group updates of a small system grow with G^2
    const int g = c.tuning.pick("lu_gemm_trail", "group", nmin, nsys, nmin >= 12000 ? 8 : 4);
    return (g >= 8 && nmin >= LU_GROUP8_MIN_N) ? 8 : 4;
}

double lu_bytes_per_unknown(int64_t n) {
    // W (2 x 2 LB floats), Y (WK floats), the FP16 panels (3 WK halves) and
    // the diagonal-block inverses (LB complex floats) per unknown
    const double wk = 2.0 * LB * (n >= LU_GROUP8_MIN_N ? LU_GROUP_MAX : 4);
    return 10.0 * wk + 16.0 * LB + 8.0 * LB + 64.0;
}

// Factors every operator of the batch and installs the preconditioner hook.
void lu_precond_setup(Context& c, GmWorkspace& ws) {
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    if (c.profiling) {
        BEM_CUDA(cudaEventCreate(&t0));
        BEM_CUDA(cudaEventCreate(&t1));
        BEM_CUDA(cudaEventRecord(t0, c.stream));
    }
    auto d = std::make_shared<LuData>();
    const int nsys = ws.bt.nsys;
    std::vector<GmView> v((size_t)nsys);
    size_t entries = 0, dm = 0, wsz = 0, psz = 0, hsz = 0;
    // split FP64 operators: each occupies two FP32 planes, of which the
    // factors copy the first (the operator's FP32 rounding) to half the offset
    const size_t fdiv = ws.bt.split_lo ? 2 : 1;
    int64_t nmin = INT64_MAX, nmax_all = 0;
    for (int s = 0; s < nsys; ++s) {
        const int64_t ns_ = ws.sys_host.empty() ? ws.bt.n : ws.sys_host[(size_t)s].n;
        nmin = std::min(nmin, ns_);
        nmax_all = std::max(nmax_all, ns_);
    }
    const int G = lu_group(c, nmin, nsys);
    const int WK = 2 * LB * G;
    d->group = G;
    for (int s = 0; s < nsys; ++s) {
        v[(size_t)s] = ws.sys_host.empty() ? gm_view(ws.bt, s) : GmView{};
        if (!ws.sys_host.empty()) {
            const GmSys& q = ws.sys_host[(size_t)s];
            v[(size_t)s].n = q.n;
            v[(size_t)s].lda = q.lda;
            v[(size_t)s].a = q.a_off;
        }
        entries = std::max(entries, v[(size_t)s].a / fdiv + (size_t)v[(size_t)s].lda * v[(size_t)s].n);
        const int nb = (int)((v[(size_t)s].n + LB - 1) / LB);
        dm += (size_t)nb * LB * LB;
        wsz += (size_t)2 * v[(size_t)s].n * (2 * LB);
        psz += (size_t)2 * (2 * LB) * (2 * LB) + (size_t)WK * v[(size_t)s].n;
        hsz += (size_t)3 * v[(size_t)s].n * WK;  // W16 (2n x WK) and Y16 (n x WK)
        d->nblk_max = std::max(d->nblk_max, nb);
    }
    // the factors, block inverses and panel workspace live in grow-only
    // buffers of the context
    c.w_lu_F.ensure(sizeof(float2) * entries);
    c.w_lu_D.ensure(sizeof(float2) * std::max<size_t>(dm, 1));
    c.w_lu_W.ensure(sizeof(float) * std::max<size_t>(wsz, 4));
    c.w_lu_P.ensure(sizeof(float) * std::max<size_t>(psz, 4));
    c.w_lu_H.ensure(sizeof(__half) * std::max<size_t>(hsz, 8));
    // the FP16 copy of U12 is scaled by 2^10 over the operator's Frobenius
    // norm (a bound on its largest entry; a power of two, so exact)
    std::vector<double> anorm((size_t)nsys);
    BEM_CUDA(cudaMemcpyAsync(anorm.data(), ws.anorm, sizeof(double) * nsys, cudaMemcpyDeviceToHost, c.stream));
    c.sync();
    if (ws.bt.split_lo) {
        // one copy per distinct operator (several right-hand sides share one)
        for (int s = 0; s < nsys; ++s) {
            bool first = true;
            for (int o = 0; o < s && first; ++o) first = v[(size_t)o].a != v[(size_t)s].a;
            require(v[(size_t)s].a % 2 == 0, "LU: split operator offset", BEM_ERR_CUDA);
            if (first)
                BEM_CUDA(cudaMemcpyAsync(c.w_lu_F.as<float2>() + v[(size_t)s].a / 2,
                                         static_cast<const float2*>(ws.bt.A) + v[(size_t)s].a,
                                         sizeof(float2) * (size_t)v[(size_t)s].lda * v[(size_t)s].n,
                                         cudaMemcpyDeviceToDevice, c.stream));
        }
    } else if (ws.fp32) {
        BEM_CUDA(cudaMemcpyAsync(c.w_lu_F.p, ws.bt.A, sizeof(float2) * entries, cudaMemcpyDeviceToDevice, c.stream));
    } else {
        // FP64 operator (refined form): factor its FP32 rounding
        const unsigned g = (unsigned)std::min<size_t>((entries + 255) / 256, (size_t)1 << 20);
        lu_round_kernel<<<g, 256, 0, c.stream>>>(static_cast<const double2*>(ws.bt.A), entries,
                                                 c.w_lu_F.as<float2>());
        BEM_CHECK_LAUNCH(&c);
    }
    // systems sharing an operator (several right-hand sides) share its factors
    std::vector<int> owner((size_t)nsys);
    for (int s = 0; s < nsys; ++s) {
        owner[(size_t)s] = s;
        for (int o = 0; o < s; ++o)
            if (owner[(size_t)o] == o && v[(size_t)o].a == v[(size_t)s].a) {
                owner[(size_t)s] = o;
                break;
            }
    }
    d->sys.resize((size_t)nsys);
    constexpr int NMAP = 7;
    d->maps.ensure(sizeof(CUtensorMap) * NMAP * nsys);
    std::vector<CUtensorMap> maps((size_t)(NMAP * nsys));
    const PFN_cuTensorMapEncodeTiled_v12000 encode = tensor_map_encoder();
    // a 2-D FP32 tensor map with 128-byte swizzled boxes of 32 floats x rows
    auto map2d = [&](CUtensorMap* m, const void* base, uint64_t inner, uint64_t outer, uint64_t stride_floats,
                     uint32_t box_rows, const char* what) {
        const cuuint64_t dims[2] = {(cuuint64_t)inner, (cuuint64_t)outer};
        const cuuint64_t strides[1] = {(cuuint64_t)(stride_floats * sizeof(float))};
        const cuuint32_t box[2] = {(cuuint32_t)GK, (cuuint32_t)box_rows};
        const cuuint32_t es[2] = {1, 1};
        const CUresult r = encode(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(base), dims, strides, box,
                                  es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        require(r == CUDA_SUCCESS, std::string("LU: tensor map of ") + what);
    };
    // the same for FP16 with boxes of 64 halves x rows (128-byte rows)
    auto map2d16 = [&](CUtensorMap* m, const void* base, uint64_t inner, uint64_t outer, uint64_t stride_halves,
                       uint32_t box_rows, const char* what) {
        const cuuint64_t dims[2] = {(cuuint64_t)inner, (cuuint64_t)outer};
        const cuuint64_t strides[1] = {(cuuint64_t)(stride_halves * sizeof(__half))};
        const cuuint32_t box[2] = {(cuuint32_t)GK16, (cuuint32_t)box_rows};
        const cuuint32_t es[2] = {1, 1};
        const CUresult r = encode(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<void*>(base), dims, strides, box,
                                  es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        require(r == CUDA_SUCCESS, std::string("LU: tensor map of ") + what);
    };
    size_t od = 0, ow = 0, op = 0, oh = 0;
    for (int s = 0; s < nsys; ++s) {
        LuSys& L = d->sys[(size_t)s];
        if (owner[(size_t)s] != s) {
            L = d->sys[(size_t)owner[(size_t)s]];
            continue;
        }
        L.F = c.w_lu_F.as<float2>() + v[(size_t)s].a / fdiv;
        L.Dm = c.w_lu_D.as<float2>() + od;
        L.W = c.w_lu_W.as<float>() + ow;
        L.n = v[(size_t)s].n;
        L.ld = v[(size_t)s].lda;
        L.nblk = (int)((L.n + LB - 1) / LB);
        L.Li = c.w_lu_P.as<float>() + op;
        L.UiT = L.Li + (2 * LB) * (2 * LB);
        L.Y = L.UiT + (2 * LB) * (2 * LB);
        L.W16 = c.w_lu_H.as<__half>() + oh;
        L.Y16 = L.W16 + (size_t)2 * L.n * WK;
        const double an = anorm[(size_t)s];
        const int e = (std::isfinite(an) && an > 0) ? std::max(-100, std::min(100, 10 - (int)std::ceil(std::log2(an))))
                                                    : 0;
        L.ysc = std::ldexp(1.0f, e);
        L.yinv = std::ldexp(1.0f, -e);
        L.wk = WK;
        od += (size_t)L.nblk * LB * LB;
        ow += (size_t)2 * L.n * (2 * LB);
        op += (size_t)2 * (2 * LB) * (2 * LB) + (size_t)WK * L.n;
        oh += (size_t)3 * L.n * WK;
        CUtensorMap* ms = maps.data() + (size_t)NMAP * s;
        map2d(ms + 0, L.W, 2 * LB, 2 * L.n, 2 * LB, GM, "the panel workspace");        // W
        map2d(ms + 1, L.F, 2 * L.n, L.n, 2 * L.ld, GN, "the factors");                 // F, natural real view
        map2d(ms + 2, L.Y, WK, L.n, WK, GN, "the row panel");                          // Y
        map2d(ms + 3, L.Li, 2 * LB, 2 * LB, 2 * LB, GM, "the lower inverse");          // Li
        map2d(ms + 4, L.UiT, 2 * LB, 2 * LB, 2 * LB, GN, "the upper inverse");         // UiT
        map2d16(ms + 5, L.W16, WK, 2 * L.n, WK, GM, "the FP16 column panels");       // W16
        map2d16(ms + 6, L.Y16, WK, L.n, WK, GN, "the FP16 row panels");              // Y16
        CUtensorMap* md = d->maps.as<CUtensorMap>() + (size_t)NMAP * s;
        L.tmW = md + 0;
        L.tmF = md + 1;
        L.tmY = md + 2;
        L.tmL = md + 3;
        L.tmU = md + 4;
        L.tmW16 = md + 5;
        L.tmY16 = md + 6;
    }
    BEM_CUDA(cudaMemcpyAsync(d->maps.p, maps.data(), sizeof(CUtensorMap) * maps.size(), cudaMemcpyHostToDevice,
                             c.stream));
    // the factorization plan: block steps in groups of LU_GROUP (delayed
    // update).  Before step k + j of the group (j > 0) its block column (from
    // the diagonal block down) and block row receive the updates of steps
    // k .. k + j - 1 at once (K = 256 j); then its diagonal block and panels.
    // After the group, one K = 256 LU_GROUP update of the rest with every
    // step's panels side by side: A22 is read and written once per group.
    auto plan = [&](LuData::Kind kind, int ks, int kw, int woff, int yoff, int nchunks,
                    const std::vector<Entry>& e) {
        LuData::Launch l{kind, ks, kw, woff, yoff, nchunks, add_segment(*d, e)};
        if (l.seg.ctas) d->plan.push_back(l);
    };
    for (int k = 0; k < d->nblk_max; k += G) {
        const int64_t ktw = (int64_t)(k + 1) * LB;  // trailing origin of the group: W row 0
        for (int j = 0; j < G; ++j) {
            const int st = k + j;
            std::vector<Entry> thin, diag, expd, l21, u12, copy;
            for (int s = 0; s < nsys; ++s) {
                const LuSys& L = d->sys[(size_t)s];
                if (L.nblk <= st || owner[(size_t)s] != s) continue;  // factored once per operator
                const int64_t kts = (int64_t)(st + 1) * LB, mts = L.n - kts, mtw = L.n - ktw;
                if (j > 0) {
                    const int64_t c0 = (int64_t)st * LB;
                    thin.push_back(trail_entry(s, 2 * (j - 1) * LB, 2 * mtw, c0, std::min<int64_t>(c0 + LB, L.n)));
                    thin.push_back(trail_entry(s, 2 * (j - 1) * LB, 2 * j * LB, c0 + LB, L.n));
                }
                diag.push_back(Entry{s, 1, 0, 0, 0, 0, 0});
                if (mts <= 0) continue;  // the system's last block
                expd.push_back(Entry{s, (mts + 63) / 64, 0, 0, 0, 0, 0});
                l21.push_back(Entry{s, (2 * mts + GM - 1) / GM, 0, 2 * j * LB, 2 * mtw, 0, 0});
                u12.push_back(Entry{s, 2 * ((mts + GN - 1) / GN), 0, 0, 0, kts, L.n});
                copy.push_back(Entry{s, (mts + 31) / 32, 0, 0, 0, 0, 0});
            }
            plan(LuData::TRAIL, st, k, 0, 0, GCHUNKS16 * j, thin);
            plan(LuData::DIAG, st, k, 0, 0, 0, diag);
            plan(LuData::EXPAND, st, k, 2 * LB * j, 0, 0, expd);
            plan(LuData::L21, st, k, 2 * LB * j, 0, GCHUNKS, l21);
            plan(LuData::U12, st, k, 0, 2 * LB * j, GCHUNKS, u12);
            plan(LuData::COPY, st, k, 0, 2 * LB * j, 0, copy);
        }
        std::vector<Entry> rest;
        for (int s = 0; s < nsys; ++s) {
            const LuSys& L = d->sys[(size_t)s];
            const int64_t c0 = (int64_t)(k + G) * LB;
            if (owner[(size_t)s] != s || c0 >= L.n) continue;
            rest.push_back(trail_entry(s, 2 * (G - 1) * LB, 2 * (L.n - ktw), c0, L.n));
        }
        plan(LuData::TRAIL, k + G - 1, k, 0, 0, GCHUNKS16 * G, rest);
    }
    // substitution tickets: forward rows by ascending block, then backward
    // rows by descending block, the groups interleaved.  A group is up to
    // TS_MAXR consecutive systems sharing one operator (several right-hand
    // sides): one ticket streams the factors once for all of them.
    {
        std::vector<int> gs, gn, fo;  // group: first system, systems, flag offset
        int nf = 1;                   // [0] is the ticket counter
        for (int s = 0; s < nsys;) {
            int r = 1;
            while (r < TS_MAXR && s + r < nsys && owner[(size_t)(s + r)] == owner[(size_t)s]) ++r;
            gs.push_back(s);
            gn.push_back(r);
            fo.push_back(nf);
            nf += 2 * d->sys[(size_t)s].nblk;
            d->trsv_r = std::max(d->trsv_r, r);
            s += r;
        }
        if (d->trsv_r == 3) d->trsv_r = TS_MAXR;
        std::vector<LuTicket> tk;
        for (int ph = 0; ph < 2; ++ph)
            for (int t = 0; t < d->nblk_max; ++t)
                for (size_t q = 0; q < gs.size(); ++q) {
                    const int nb = d->sys[(size_t)gs[q]].nblk;
                    if (t < nb) tk.push_back(LuTicket{gs[q], gn[q], ph, ph == 0 ? t : nb - 1 - t, fo[q]});
                }
        d->ntickets = (int)tk.size();
        d->nflags = nf;
        d->tickets.ensure(sizeof(LuTicket) * std::max<size_t>(tk.size(), 1));
        d->flags.ensure(sizeof(int) * (size_t)nf);
        BEM_CUDA(cudaMemcpyAsync(d->tickets.p, tk.data(), sizeof(LuTicket) * tk.size(), cudaMemcpyHostToDevice,
                                 c.stream));
        int per_sm = 1, nsm_ = 0;
        const void* kfn = d->trsv_r == 1   ? (const void*)lu_trsv_kernel<1>
                          : d->trsv_r == 2 ? (const void*)lu_trsv_kernel<2>
                                           : (const void*)lu_trsv_kernel<TS_MAXR>;
        BEM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, TS_THREADS, 0));
        BEM_CUDA(cudaDeviceGetAttribute(&nsm_, cudaDevAttrMultiProcessorCount, c.device));
        d->trsv_grid = std::max(1, std::min(d->ntickets, std::max(1, per_sm) * nsm_));
    }
    d->sysbuf.ensure(sizeof(LuSys) * nsys);
    d->work.ensure(sizeof(LuWork) * std::max<size_t>(d->host.size(), 1));
    d->info.ensure(sizeof(int));
    BEM_CUDA(cudaMemcpyAsync(d->sysbuf.p, d->sys.data(), sizeof(LuSys) * nsys, cudaMemcpyHostToDevice, c.stream));
    BEM_CUDA(cudaMemcpyAsync(d->work.p, d->host.data(), sizeof(LuWork) * d->host.size(), cudaMemcpyHostToDevice,
                             c.stream));
    BEM_CUDA(cudaMemsetAsync(d->info.p, 0, sizeof(int), c.stream));
    int* err = device_err(c);
    BEM_CUDA(cudaMemsetAsync(err, 0, sizeof(int), c.stream));
    const size_t diag_smem = sizeof(float2) * LB * DIAG_TS, expand_smem = sizeof(float2) * 65 * LB;
    BEM_CUDA(cudaFuncSetAttribute(lu_diag_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)diag_smem));
    BEM_CUDA(cudaFuncSetAttribute(lu_expand_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)expand_smem));
    BEM_CUDA(cudaFuncSetAttribute(lu_gemm_kernel<G_TRAIL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G_SMEM));
    BEM_CUDA(cudaFuncSetAttribute(lu_gemm_kernel<G_U12>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G_SMEM));
    BEM_CUDA(cudaFuncSetAttribute(lu_gemm_kernel<G_L21>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G_SMEM));
    const LuSys* sys = d->sysbuf.as<LuSys>();
    const LuWork* wk = d->work.as<LuWork>();
    int nsm = 0;
    BEM_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c.device));  // persistent grids
    // with profiling: CUDA events around every launch, summed per kind
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    float tsum[6] = {0, 0, 0, 0, 0, 0};  // per launch kind
    if (c.profiling) {
        BEM_CUDA(cudaEventCreate(&ev0));
        BEM_CUDA(cudaEventCreate(&ev1));
    }
    auto persistent = [&](int64_t ctas) { return (unsigned)std::min<int64_t>(ctas, nsm); };
    // tile raster of the trailing updates (super-blocks of sb_r x sb_c tiles)
    // (keyed by the largest operator and the number of factored operators)
    int64_t nfact = 0, nmax = 0;
    for (int s = 0; s < nsys; ++s) {
        nfact += owner[(size_t)s] == s;
        nmax = std::max(nmax, d->sys[(size_t)s].n);
    }
    const int sb_r = std::max(1, std::min(65535, c.tuning.pick("lu_gemm_trail", "sb_r", nmax, nfact, 8)));
    const int sb_c = std::max(1, std::min(65535, c.tuning.pick("lu_gemm_trail", "sb_c", nmax, nfact, 32)));
    const int raster = (sb_r << 16) | sb_c;
    for (const LuData::Launch& l : d->plan) {
        const LuData::Seg& sg = l.seg;
        if (c.profiling) BEM_CUDA(cudaEventRecord(ev0, c.stream));
        switch (l.kind) {
            case LuData::DIAG:
                lu_diag_kernel<<<(unsigned)sg.ctas, DIAG_THREADS, diag_smem, c.stream>>>(sys, wk + sg.off, l.ks,
                                                                                 d->info.as<int>());
                break;
            case LuData::EXPAND:
                lu_expand_kernel<<<(unsigned)sg.ctas, 256, expand_smem, c.stream>>>(sys, wk + sg.off, sg.count, l.ks,
                                                                                    l.kw);
                break;
            case LuData::L21:
                lu_gemm_kernel<G_L21><<<persistent(sg.ctas), GTHREADS, G_SMEM, c.stream>>>(
                    sys, wk + sg.off, sg.count, l.ks, l.kw, l.nchunks, l.woff, l.yoff, sg.ctas, raster, err);
                break;
            case LuData::U12:
                lu_gemm_kernel<G_U12><<<persistent(sg.ctas), GTHREADS, G_SMEM, c.stream>>>(
                    sys, wk + sg.off, sg.count, l.ks, l.kw, l.nchunks, l.woff, l.yoff, sg.ctas, raster, err);
                break;
            case LuData::COPY:
                lu_copy_u12_kernel<<<(unsigned)sg.ctas, 256, 0, c.stream>>>(sys, wk + sg.off, sg.count, l.ks,
                                                                            l.yoff);
                break;
            case LuData::TRAIL:
                lu_gemm_kernel<G_TRAIL><<<persistent(sg.ctas), GTHREADS, G_SMEM, c.stream>>>(
                    sys, wk + sg.off, sg.count, l.ks, l.kw, l.nchunks, l.woff, l.yoff, sg.ctas, raster, err);
                break;
        }
        BEM_CHECK_LAUNCH(&c);
        if (c.profiling) {
            BEM_CUDA(cudaEventRecord(ev1, c.stream));
            BEM_CUDA(cudaEventSynchronize(ev1));
            float ms = 0;
            BEM_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
            tsum[(int)l.kind] += ms;
        }
    }
    if (c.profiling) {
        // algorithmic work: 8 n^3 / 3 complex flop per factored operator
        double fl = 0;
        for (int s = 0; s < nsys; ++s)
            if (owner[(size_t)s] == s) fl += 8.0 / 3.0 * std::pow((double)d->sys[(size_t)s].n, 3.0);
        c.stage_add("lu_diag", tsum[LuData::DIAG], d->nblk_max, 0);
        c.stage_add("lu_panel_expand", tsum[LuData::EXPAND], d->nblk_max, 0);
        c.stage_add("lu_panel_l21", tsum[LuData::L21], d->nblk_max, 0);
        c.stage_add("lu_panel_u12", tsum[LuData::U12], d->nblk_max, 0);
        c.stage_add("lu_panel_copy", tsum[LuData::COPY], d->nblk_max, 0);
        c.stage_add("lu_gemm_trail", tsum[LuData::TRAIL], d->nblk_max, fl);
        cudaEventDestroy(ev0);
        cudaEventDestroy(ev1);
    }
    check_device_err(c);
    BEM_CUDA(cudaMemcpyAsync(&d->small_pivots, d->info.p, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    c.sync();
    if (c.profiling) {
        BEM_CUDA(cudaEventRecord(t1, c.stream));
        BEM_CUDA(cudaEventSynchronize(t1));
        float ms = 0;
        BEM_CUDA(cudaEventElapsedTime(&ms, t0, t1));
        c.stage_add("lu_setup_total", ms, 1, 0);
        cudaEventDestroy(t0);
        cudaEventDestroy(t1);
    }
    ws.zb().ensure(sizeof(double2) * gm_q_total(ws));
    ws.bt.Z = ws.zb().as<double2>();
    ws.precond = lu_hook;
    ws.precond_user = d.get();
    ws.precond_keep = d;
}

}  // namespace bem

// ---------------------------------------------------------------------------
// Instrumentation: the preconditioner's factorization and one application on
// caller-given FP32 operators, with the factors read back, so that the device
// kernels can be compared entry by entry with an FP64 LU.
using namespace bem;

extern "C" BEM_API bem_status bem_lu32_factor_apply(bem_ctx* ctx, int nsys, const int64_t* n, const int64_t* ld,
                                                    const int64_t* a_off, int64_t a_entries, const float* A,
                                                    float* F, float* D, int64_t d_entries, const bem_cplx* q,
                                                    bem_cplx* z, int* small_pivots) {
    if (!ctx || nsys < 1 || !n || !ld || !a_off || !A || a_entries <= 0) return BEM_ERR_BAD_INPUT;
    Context& c = ctx->c;
    try {
        BEM_CUDA(cudaSetDevice(c.device));
        std::vector<int64_t> ns(n, n + nsys), lds(ld, ld + nsys);
        std::vector<size_t> offs((size_t)nsys);
        int64_t dneed = 0;
        for (int s = 0; s < nsys; ++s) {
            require(ns[(size_t)s] >= 1 && lds[(size_t)s] >= ns[(size_t)s], "lu32: bad system size");
            // the production layout: leading dimension and offset multiples
            // of 64 entries (16-byte aligned tensor copies and vector loads)
            require(lds[(size_t)s] % 64 == 0 && a_off[s] % 64 == 0 && a_off[s] >= 0,
                    "lu32: leading dimensions and offsets must be multiples of 64");
            require(a_off[s] + lds[(size_t)s] * ns[(size_t)s] <= a_entries, "lu32: operator outside A");
            offs[(size_t)s] = (size_t)a_off[s];
            bool owner = true;
            for (int o = 0; o < s; ++o)
                if (a_off[o] == a_off[s]) {
                    require(ns[(size_t)o] == ns[(size_t)s] && lds[(size_t)o] == lds[(size_t)s],
                            "lu32: systems sharing an operator must have the same size");
                    owner = false;
                    break;
                }
            if (owner) dneed += (int64_t)((ns[(size_t)s] + LB - 1) / LB) * LB * LB;
        }
        require(!D || d_entries == dneed,
                "lu32: D must hold " + std::to_string(dneed) + " complex entries (128 x 128 per block)");
        DevBuf dA;
        dA.ensure(sizeof(float2) * (size_t)a_entries);
        BEM_CUDA(cudaMemcpyAsync(dA.p, A, sizeof(float2) * (size_t)a_entries, cudaMemcpyHostToDevice, c.stream));
        GmWorkspace ws;
        gm_prepare_ragged(c, ws, ns, lds, offs, 1, dA.p, true);
        gm_matrix_norms(c, ws);  // the scale of the FP16 row panels
        // every system active at Krylov step 0 (the state the application reads)
        BEM_CUDA(cudaMemsetAsync(ws.bt.st, 0, sizeof(GmState) * (size_t)nsys, c.stream));
        if (q) {
            size_t v = 0;
            for (int s = 0; s < nsys; ++s) {
                BEM_CUDA(cudaMemcpyAsync(ws.bt.Q + ws.sys_host[(size_t)s].q_off, q + v,
                                         sizeof(double2) * (size_t)ns[(size_t)s], cudaMemcpyHostToDevice, c.stream));
                v += (size_t)ns[(size_t)s];
            }
        }
        lu_precond_setup(c, ws);
        LuData& d = *static_cast<LuData*>(ws.precond_user);
        if (q && z) {
            ws.precond(c, ws, MV_Q, ws.precond_user);
            check_device_err(c);
            size_t v = 0;
            for (int s = 0; s < nsys; ++s) {
                BEM_CUDA(cudaMemcpyAsync(z + v, ws.bt.Z + ws.sys_host[(size_t)s].q_off,
                                         sizeof(double2) * (size_t)ns[(size_t)s], cudaMemcpyDeviceToHost, c.stream));
                v += (size_t)ns[(size_t)s];
            }
        }
        if (F) {
            size_t fent = 0;
            for (int s = 0; s < nsys; ++s)
                fent = std::max(fent, offs[(size_t)s] + (size_t)lds[(size_t)s] * (size_t)ns[(size_t)s]);
            BEM_CUDA(cudaMemcpyAsync(F, c.w_lu_F.p, sizeof(float2) * fent, cudaMemcpyDeviceToHost, c.stream));
        }
        if (D)
            BEM_CUDA(cudaMemcpyAsync(D, c.w_lu_D.p, sizeof(float2) * (size_t)dneed, cudaMemcpyDeviceToHost,
                                     c.stream));
        c.sync();
        if (small_pivots) *small_pivots = d.small_pivots;
        return BEM_OK;
    } catch (const Error& e) {
        c.last_error = e.what();
        return e.status;
    } catch (const std::exception& e) {
        c.last_error = e.what();
        return BEM_ERR_CUDA;
    }
}

