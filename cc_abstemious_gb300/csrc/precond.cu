// Preconditioners for the batched GMRES (flexible right preconditioning,
// Z[:, k] = M Q[:, k]).
//
// The unknowns are grouped by the leaves of the cluster tree (bounding-box
// bisection of cluster.rs, leaf size 64).  Two leaves are "near" when the
// block-tree admissibility test min(diam) <= eta * dist fails for them.
//
//  * Block-Jacobi: M = blockdiag(A_cc)^-1, the exact inverse of every diagonal
//    leaf block (Gauss-Jordan with partial pivoting, one CTA per block).
//  * Learned: M = blockdiag(A_cc)^-1 + C, where C lives on the near
//    off-diagonal leaf blocks and every entry C_ij is emitted by a 3-layer MLP
//    (16 -> 128 -> 128 -> 2, tanh, width 128) from geometry only: the pair's
//    separation scaled by the element size, both normals, the area ratio, k h
//    and the phase k r.  C_ij = s_ij (o_1 + i o_2) with s_ij = wa_j / (4 pi r).
//    Weights and activations are rounded to BF16, products accumulate in
//    FP32.  The network is trained on the GPU on operators the BEM assembles,
//    minimising E_z ||A M z - z||^2 / ||z||^2 over random probes z (relative to
//    the system's block-Jacobi value, so every wavenumber weighs alike), with
//    hand-written forward / backward kernels and Adam.  The block-Jacobi part
//    is always present, so an untrained (zero) correction is block-Jacobi.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <chrono>
#include <cstring>
#include <memory>
#include <random>

#include "common.cuh"
#include "complex.cuh"
#include "gmres.cuh"
#include "hmatrix.cuh"
#include "kernels.cuh"
#include "precond.cuh"
#include "tree.cuh"

namespace bem {

constexpr int PC_LEAF = 64;
constexpr double PC_ETA = 2.0;

// ---------------------------------------------------------------------------
// Near-field leaf patterns: the cluster trees of all bodies in one device
// pass, then per body its leaves and their near neighbours.  Several bodies
// are built on parallel host threads (each writes only its own pattern); a
// single body spreads its leaves over the threads instead.
void build_patterns(Context& c, const std::vector<const Problem*>& bodies, std::vector<NearPattern>& pats,
                    bool diag_only) {
    auto F = build_forest(c, bodies, PC_LEAF);
    pats.resize(bodies.size());
    if (bodies.size() == 1) {
        near_pattern(*F, 0, pats[0], diag_only, true);
        return;
    }
    host_parallel_for((int64_t)bodies.size(),
                      [&](int64_t b) { near_pattern(*F, (int)b, pats[(size_t)b], diag_only, false); });
}

void near_pattern(const Forest& F, int body, NearPattern& P, bool diag_only, bool parallel) {
    const int l0 = F.leaf0[(size_t)body], l1 = F.leaf0[(size_t)body + 1];
    std::vector<const TreeNode*> leaves;
    for (int l = l0; l < l1; ++l) leaves.push_back(&F.nodes[(size_t)F.leaves[(size_t)l]]);
    P.n = F.n(body);
    P.nc = (int)leaves.size();
    const int nc = P.nc;
    // the leaves are consecutive ranges of the body's cluster order
    P.cl_idx.assign(F.perm.begin() + F.pt0[(size_t)body], F.perm.begin() + F.pt0[(size_t)body + 1]);
    P.cl_off.assign(1, 0);
    for (const TreeNode* l : leaves) P.cl_off.push_back(l->end);
    auto size_of = [&](int c) { return P.cl_off[(size_t)c + 1] - P.cl_off[(size_t)c]; };
    auto each_leaf = [&](const std::function<void(int64_t)>& f) {
        if (parallel) host_parallel_for(nc, f);
        else
            for (int64_t c = 0; c < nc; ++c) f(c);
    };
    // near neighbours of every leaf (itself first, then the inadmissible
    // partners in leaf order) with their block entries and pair counts
    std::vector<std::vector<int>> near((size_t)nc);
    std::vector<int64_t> ent((size_t)nc + 1, 0), pairs((size_t)nc + 1, 0);
    each_leaf([&](int64_t c) {
        std::vector<int>& nr = near[(size_t)c];
        nr.push_back((int)c);
        const int64_t bc = size_of((int)c);
        int64_t e = bc * bc, q = 0;
        for (int d = 0; d < nc && !diag_only; ++d) {
            if (d == c) continue;
            if (!(std::fmin(leaves[(size_t)c]->diam, leaves[(size_t)d]->diam) <=
                  PC_ETA * node_distance(*leaves[(size_t)c], *leaves[(size_t)d]))) {
                nr.push_back(d);
                e += bc * size_of(d);
                q += bc * size_of(d);
            }
        }
        ent[(size_t)c + 1] = e;
        pairs[(size_t)c + 1] = q;
    });
    P.nb_off.assign((size_t)nc + 1, 0);
    for (int c = 0; c < nc; ++c) {
        P.nb_off[(size_t)c + 1] = P.nb_off[(size_t)c] + (int32_t)near[(size_t)c].size();
        ent[(size_t)c + 1] += ent[(size_t)c];
        pairs[(size_t)c + 1] += pairs[(size_t)c];
    }
    P.entries = ent[(size_t)nc];
    P.npairs = pairs[(size_t)nc];
    P.nb_d.resize((size_t)P.nb_off[(size_t)nc]);
    P.nb_blk.resize((size_t)P.nb_off[(size_t)nc]);
    P.pair_i.resize((size_t)P.npairs);
    P.pair_j.resize((size_t)P.npairs);
    P.pair_dst.resize((size_t)P.npairs);
    // blocks stored back to back in (leaf, neighbour) order, each b_c x b_d
    // column-major; the pairs of the off-diagonal ones in storage order
    each_leaf([&](int64_t c) {
        const int64_t bc = size_of((int)c), oc = P.cl_off[(size_t)c];
        int64_t e = ent[(size_t)c], q = pairs[(size_t)c];
        int32_t t = P.nb_off[(size_t)c];
        for (int d : near[(size_t)c]) {
            const int64_t bd = size_of(d), od = P.cl_off[(size_t)d];
            P.nb_d[(size_t)t] = d;
            P.nb_blk[(size_t)t] = e;
            ++t;
            if (d != c)
                for (int64_t jj = 0; jj < bd; ++jj)
                    for (int64_t ii = 0; ii < bc; ++ii, ++q) {
                        P.pair_i[(size_t)q] = (int32_t)P.cl_idx[(size_t)(oc + ii)];
                        P.pair_j[(size_t)q] = (int32_t)P.cl_idx[(size_t)(od + jj)];
                        P.pair_dst[(size_t)q] = e + jj * bc + ii;
                    }
            e += bc * bd;
        }
    });
}

// ---------------------------------------------------------------------------
// Exact inverse of every diagonal leaf block, [A_cc | I] reduced by
// Gauss-Jordan with partial pivoting in FP32, one CTA per (block, system).
struct PcDev {
    const int64_t *cl_off, *cl_idx, *nb_blk;
    const int32_t *nb_off, *nb_d;
    const float2* M;
    size_t Mstride;
    int offdiag, nc;
    // several bodies in one batch: body of each system, first leaf of each
    // body, offset of each system's blocks in M (all nullptr: one body)
    const int32_t *sys_body, *body_leaf0;
    const size_t* sys_moff;
    // learned form: per system, whether its correction is used (nullptr: all);
    // block-Jacobi alone where the correction did not lower the probe residual
    const int8_t* sys_off;
};

// Leaf index of the c-th leaf of system s's body, or -1 past its last leaf.
__device__ __forceinline__ int pc_leaf(const PcDev& pc, int s, int c) {
    if (!pc.sys_body) return c < pc.nc ? c : -1;
    const int b = pc.sys_body[s];
    const int l0 = pc.body_leaf0[b];
    return c < pc.body_leaf0[b + 1] - l0 ? l0 + c : -1;
}

__device__ __forceinline__ size_t pc_moff(const PcDev& pc, int s) {
    return pc.sys_moff ? pc.sys_moff[s] : (size_t)s * pc.Mstride;
}

template <typename T>
__global__ void __launch_bounds__(256) pc_diag_inverse_kernel(const T* __restrict__ A, int64_t lda, size_t mstride,
                                                              const GmSys* __restrict__ sys, PcDev pc,
                                                              float2* __restrict__ M) {
    extern __shared__ float2 aug[];  // b x 2b, row-major
    __shared__ int s_piv;
    __shared__ float2 fcol[PC_LEAF];  // elimination factors of the current column
    const int s = blockIdx.y;
    const int c = pc_leaf(pc, s, blockIdx.x);
    if (c < 0) return;
    const int64_t* cl_off = pc.cl_off;
    const int64_t* cl_idx = pc.cl_idx;
    const int64_t o = cl_off[c];
    const int b = (int)(cl_off[c + 1] - o);
    const int w = 2 * b;
    if (sys) lda = sys[s].lda;
    const T* As = A + (sys ? sys[s].a_off : (size_t)s * mstride);
    for (int t = threadIdx.x; t < b * b; t += blockDim.x) {
        int i = t % b, j = t / b;
        T v = As[cl_idx[o + j] * lda + cl_idx[o + i]];
        aug[i * w + j] = make_float2((float)v.x, (float)v.y);
        aug[i * w + b + j] = make_float2(i == j ? 1.f : 0.f, 0.f);
    }
    __syncthreads();
    for (int col = 0; col < b; ++col) {
        if (threadIdx.x == 0) {
            int best = col;
            float bv = -1.f;
            for (int r = col; r < b; ++r) {
                float v = fabsf(aug[r * w + col].x) + fabsf(aug[r * w + col].y);
                if (v > bv) { bv = v; best = r; }
            }
            s_piv = best;
        }
        __syncthreads();
        const int pr = s_piv;
        if (pr != col)
            for (int t = threadIdx.x; t < w; t += blockDim.x) {
                float2 a = aug[col * w + t];
                aug[col * w + t] = aug[pr * w + t];
                aug[pr * w + t] = a;
            }
        __syncthreads();
        const float2 d = aug[col * w + col];
        const float dn = d.x * d.x + d.y * d.y;
        const float2 inv = dn > 0.f ? make_float2(d.x / dn, -d.y / dn) : make_float2(0.f, 0.f);
        __syncthreads();
        for (int t = threadIdx.x; t < w; t += blockDim.x) aug[col * w + t] = fmul(aug[col * w + t], inv);
        for (int r = threadIdx.x; r < b; r += blockDim.x) fcol[r] = aug[r * w + col];
        __syncthreads();
        for (int t = threadIdx.x; t < b * w; t += blockDim.x) {
            int r = t / w, j = t % w;
            if (r == col) continue;
            float2 f = fcol[r];
            float2 v = aug[r * w + j];
            float2 u = aug[col * w + j];
            aug[r * w + j] = make_float2(v.x - (f.x * u.x - f.y * u.y), v.y - (f.x * u.y + f.y * u.x));
        }
        __syncthreads();
        // the pivot column of the other rows was consumed; zero it for clarity
    }
    float2* Mo = M + pc_moff(pc, s) + pc.nb_blk[pc.nb_off[c]];  // first neighbour is the block itself
    for (int t = threadIdx.x; t < b * b; t += blockDim.x) {
        int i = t % b, j = t / b;
        Mo[(size_t)j * b + i] = aug[i * w + b + j];
    }
}

// z[rows of c] = sum over near d of M_cd q[rows of d]; one CTA per (leaf, system).
__device__ __forceinline__ void pc_block_apply(int c, const int64_t* cl_off, const int64_t* cl_idx,
                                               const int32_t* nb_off, const int32_t* nb_d, const int64_t* nb_blk,
                                               const float2* Ms, const double2* q, double2* z, int use_offdiag) {
    __shared__ double2 qs[PC_LEAF];
    const int64_t oc = cl_off[c];
    const int bc = (int)(cl_off[c + 1] - oc);
    double2 acc = make_double2(0, 0);
    const int i = threadIdx.x;
    const int nend = use_offdiag ? nb_off[c + 1] : nb_off[c] + 1;
    for (int t = nb_off[c]; t < nend; ++t) {
        const int d = nb_d[t];
        const int64_t od = cl_off[d];
        const int bd = (int)(cl_off[d + 1] - od);
        __syncthreads();
        if (i < bd) qs[i] = q[cl_idx[od + i]];
        __syncthreads();
        if (i < bc) {
            const float2* blk = Ms + nb_blk[t];
            for (int j = 0; j < bd; ++j) {
                float2 m = blk[(size_t)j * bc + i];
                cfma(acc, make_double2(m.x, m.y), qs[j]);
            }
        }
    }
    if (i < bc) z[cl_idx[oc + i]] = acc;
}

__global__ void __launch_bounds__(PC_LEAF) pc_apply_gmres_kernel(PcDev pc, GmBatch bt) {
    const int s = blockIdx.y;
    const GmState& st = bt.st[s];
    if (!gm_apply_active(bt, st, MV_Q)) return;
    const int c = pc_leaf(pc, s, blockIdx.x);
    if (c < 0) return;
    const GmView g = gm_view(bt, s);
    const double2* q = bt.Q + g.q + (size_t)st.k * g.n;
    double2* z = bt.Z + g.q + (size_t)st.k * g.n;
    const int off = pc.offdiag && (!pc.sys_off || pc.sys_off[s]);
    pc_block_apply(c, pc.cl_off, pc.cl_idx, pc.nb_off, pc.nb_d, pc.nb_blk, pc.M + pc_moff(pc, s), q, z, off);
}

// Probe form: Y[:, q] = M_s Z[:, q] for nprobe vectors (training).
__global__ void __launch_bounds__(PC_LEAF) pc_apply_probes_kernel(PcDev pc, int s, const double2* __restrict__ Zp,
                                                                  double2* __restrict__ Yp, int64_t n) {
    const int q = blockIdx.y;
    const int c = pc_leaf(pc, s, blockIdx.x);
    if (c < 0) return;
    pc_block_apply(c, pc.cl_off, pc.cl_idx, pc.nb_off, pc.nb_d, pc.nb_blk, pc.M + pc_moff(pc, s),
                   Zp + (size_t)q * n, Yp + (size_t)q * n, pc.offdiag);
}

// ---------------------------------------------------------------------------
// MLP.  Parameters (FP32 master copy): W1 [128][16], b1 [128], W2 [128][128],
// b2 [128], W3 [2][128], b3 [2].
constexpr int NF = 16, NH = 128, NO = 2;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + NH * NF, OFF_W2 = OFF_B1 + NH, OFF_B2 = OFF_W2 + NH * NH,
              OFF_W3 = OFF_B2 + NH, OFF_B3 = OFF_W3 + NO * NH, NPARAM = OFF_B3 + NO;

__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16(x)); }
__device__ __forceinline__ float tanh_act(float x) { return tanhf(x); }

// Pair features (geometry and ka only) and the output scale.  The
// coordinate differences are taken in FP64 (near pairs share their leading
// digits), everything after in FP32: every feature is rounded to BF16 and
// the scale multiplies an FP32 entry.  One pair per thread, its 16 features
// written as four 16-byte stores.
__global__ void pc_features_kernel(int64_t P, const int32_t* __restrict__ pi, const int32_t* __restrict__ pj,
                                   int64_t npad, const double* __restrict__ geo, double k, float* __restrict__ F,
                                   float* __restrict__ scale) {
    int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= P) return;
    const int64_t i = pi[p], j = pj[p];
    const float dx = (float)(geo[GX * npad + j] - geo[GX * npad + i]);
    const float dy = (float)(geo[GY * npad + j] - geo[GY * npad + i]);
    const float dz = (float)(geo[GZ * npad + j] - geo[GZ * npad + i]);
    const float r = sqrtf(dx * dx + dy * dy + dz * dz);
    const float ai = (float)geo[GAREA * npad + i], aj = (float)geo[GAREA * npad + j];
    const float h = sqrtf(ai), hinv = 1.0f / h;
    const float kf = (float)k;
    float sn, cs;
    sincosf(kf * r, &sn, &cs);
    float f[NF] = {dx * hinv, dy * hinv, dz * hinv, r * hinv,
                   (float)geo[GNX * npad + i], (float)geo[GNY * npad + i], (float)geo[GNZ * npad + i],
                   (float)geo[GNX * npad + j], (float)geo[GNY * npad + j], (float)geo[GNZ * npad + j],
                   aj / ai, kf * h, cs, sn, h / r, 1.0f};
    float4* out = reinterpret_cast<float4*>(F + p * NF);
#pragma unroll
    for (int t = 0; t < NF / 4; ++t)
        out[t] = make_float4(bf16r(f[4 * t]), bf16r(f[4 * t + 1]), bf16r(f[4 * t + 2]), bf16r(f[4 * t + 3]));
    scale[p] = (float)geo[GWA * npad + j] / (4.0f * 3.14159265358979f * r);
}

// C = act(op(A) op(B) + bias) (+ C when accumulate).  Row-major storage;
// op(A): M x K stored [M][K] (TA = 0) or [K][M] (TA = 1); op(B): K x N stored
// [K][N] (TB = 0) or [N][K] (TB = 1).  128 x 128 tile, 8 x 8 per thread,
// FP32 accumulation.  With split > 1 the K range is split over gridDim.z and
// the results are added atomically (weight gradients).
constexpr int GB_M = 128, GB_N = 128, GB_K = 8;
template <int TA, int TB>
__global__ void __launch_bounds__(256) mlp_gemm_kernel(int64_t M, int64_t N, int64_t K, const float* __restrict__ A,
                                                       const float* __restrict__ B, float* __restrict__ C,
                                                       const float* __restrict__ bias, int act, int round_bf16,
                                                       int atomic) {
    __shared__ float As[GB_K][GB_M + 4];
    __shared__ float Bs[GB_K][GB_N + 4];
    const int64_t m0 = (int64_t)blockIdx.x * GB_M, n0 = (int64_t)blockIdx.y * GB_N;
    const int64_t kchunk = (K + gridDim.z - 1) / gridDim.z;
    const int64_t kb = (int64_t)blockIdx.z * kchunk, ke = min(K, kb + kchunk);
    const int tr = threadIdx.x / 16, tc = threadIdx.x % 16;
    float acc[8][8];
#pragma unroll
    for (int a = 0; a < 8; ++a)
#pragma unroll
        for (int b = 0; b < 8; ++b) acc[a][b] = 0.f;
    for (int64_t k0 = kb; k0 < ke; k0 += GB_K) {
        for (int t = threadIdx.x; t < GB_K * GB_M; t += 256) {
            int kk = TA ? t / GB_M : t % GB_K, mm = TA ? t % GB_M : t / GB_K;
            int64_t gm = m0 + mm, gk = k0 + kk;
            float v = 0.f;
            if (gm < M && gk < ke) v = TA ? A[gk * M + gm] : A[gm * K + gk];
            As[kk][mm] = v;
        }
        for (int t = threadIdx.x; t < GB_K * GB_N; t += 256) {
            int kk = TB ? t % GB_K : t / GB_N, nn = TB ? t / GB_K : t % GB_N;
            int64_t gn = n0 + nn, gk = k0 + kk;
            float v = 0.f;
            if (gn < N && gk < ke) v = TB ? B[gn * K + gk] : B[gk * N + gn];
            Bs[kk][nn] = v;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < GB_K; ++kk) {
            float av[8], bv[8];
#pragma unroll
            for (int a = 0; a < 8; ++a) av[a] = As[kk][tr + 16 * a];
#pragma unroll
            for (int b = 0; b < 8; ++b) bv[b] = Bs[kk][tc + 16 * b];
#pragma unroll
            for (int a = 0; a < 8; ++a)
#pragma unroll
                for (int b = 0; b < 8; ++b) acc[a][b] = fmaf(av[a], bv[b], acc[a][b]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int a = 0; a < 8; ++a) {
        const int64_t gm = m0 + tr + 16 * a;
        if (gm >= M) continue;
#pragma unroll
        for (int b = 0; b < 8; ++b) {
            const int64_t gn = n0 + tc + 16 * b;
            if (gn >= N) continue;
            float v = acc[a][b];
            if (atomic) {
                atomicAdd(&C[gm * N + gn], v);
                continue;
            }
            if (bias) v += bias[gn];
            if (act == 1) v = tanh_act(v);
            if (round_bf16) v = bf16r(v);
            C[gm * N + gn] = v;
        }
    }
}

template <int TA, int TB>
static void gemm(Context& c, int64_t M, int64_t N, int64_t K, const float* A, const float* B, float* C,
                 const float* bias, int act, int round_bf16, int split = 1) {
    dim3 grid((unsigned)((M + GB_M - 1) / GB_M), (unsigned)((N + GB_N - 1) / GB_N), (unsigned)split);
    mlp_gemm_kernel<TA, TB><<<grid, 256, 0, c.stream>>>(M, N, K, A, B, C, bias, act, round_bf16, split > 1 ? 1 : 0);
    BEM_CHECK_LAUNCH(&c);
}

// BF16 copy of the weights (kept as FP32 values) used by the forward pass.
__global__ void round_params_kernel(int n, const float* __restrict__ w, float* __restrict__ wb) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) wb[t] = bf16r(w[t]);
}

// Learned entries into the block storage of one system.
__global__ void pc_write_learned_kernel(int64_t P, const float* __restrict__ O, const float* __restrict__ scale,
                                        const int64_t* __restrict__ dst, float2* __restrict__ M) {
    int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= P) return;
    M[dst[p]] = make_float2(scale[p] * O[2 * p], scale[p] * O[2 * p + 1]);
}

void mlp_forward(Context& c, const LearnedNet& net, int64_t P, const float* F, float* H1, float* H2, float* O) {
    const float* wb = net.wbf.as<float>();
    gemm<0, 1>(c, P, NH, NF, F, wb + OFF_W1, H1, wb + OFF_B1, 1, 1);
    gemm<0, 1>(c, P, NH, NH, H1, wb + OFF_W2, H2, wb + OFF_B2, 1, 1);
    gemm<0, 1>(c, P, NO, NH, H2, wb + OFF_W3, O, wb + OFF_B3, 0, 0);
}

// ---------------------------------------------------------------------------
// Training kernels.
__device__ __forceinline__ uint64_t mix64(uint64_t x) {
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdULL;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ULL;
    x ^= x >> 33;
    return x;
}

// Complex Gaussian probes (Box-Muller on a counter hash).
__global__ void probes_kernel(int64_t total, uint64_t seed, double2* __restrict__ Z) {
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= total) return;
    uint64_t a = mix64(seed ^ (2 * (uint64_t)t + 1)), b = mix64(seed + 0x9E3779B97F4A7C15ULL * (uint64_t)(t + 7));
    double u1 = ((a >> 11) + 1) * (1.0 / 9007199254740993.0), u2 = (b >> 11) * (1.0 / 9007199254740992.0);
    double rr = sqrt(-2.0 * log(u1));
    Z[t] = make_double2(rr * cos(6.283185307179586 * u2), rr * sin(6.283185307179586 * u2));
}

// Y[:, q] = A X[:, q] (conj = 0) or A^H X[:, q] (conj = 1), FP32 operator,
// column-major with leading dimension lda.  One CTA per (row block or column, probe).
__global__ void probe_matvec_kernel(int64_t n, const float2* __restrict__ A, int64_t lda, const double2* __restrict__ X,
                                    double2* __restrict__ Y, int conj) {
    const int q = blockIdx.y;
    const double2* x = X + (size_t)q * n;
    double2* y = Y + (size_t)q * n;
    if (!conj) {
        int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
        if (i >= n) return;
        double2 acc = make_double2(0, 0);
        for (int64_t j = 0; j < n; ++j) {
            float2 a = A[j * lda + i];
            cfma(acc, make_double2(a.x, a.y), x[j]);
        }
        y[i] = acc;
    } else {
        // y_j = sum_i conj(A_ij) x_i: one warp per column j
        int64_t j = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / 32;
        int lane = threadIdx.x & 31;
        if (j >= n) return;
        double ax = 0, ay = 0;
        for (int64_t i = lane; i < n; i += 32) {
            float2 a = A[j * lda + i];
            double2 v = x[i];
            ax += a.x * v.x + a.y * v.y;
            ay += a.x * v.y - a.y * v.x;
        }
        for (int o = 16; o > 0; o >>= 1) {
            ax += __shfl_down_sync(0xffffffffu, ax, o);
            ay += __shfl_down_sync(0xffffffffu, ay, o);
        }
        if (lane == 0) y[j] = make_double2(ax, ay);
    }
}

// R = W - Z, per-probe |R|^2 and |Z|^2 partials (loss).
__global__ void probe_residual_kernel(int64_t total, const double2* __restrict__ W, const double2* __restrict__ Z,
                                      double2* __restrict__ R, double* __restrict__ acc) {
    __shared__ double sr[256], sz[256];
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    double a = 0, b = 0;
    if (t < total) {
        double2 r = csub(W[t], Z[t]);
        R[t] = r;
        a = r.x * r.x + r.y * r.y;
        b = Z[t].x * Z[t].x + Z[t].y * Z[t].y;
    }
    sr[threadIdx.x] = a;
    sz[threadIdx.x] = b;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            sr[threadIdx.x] += sr[threadIdx.x + o];
            sz[threadIdx.x] += sz[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        atomicAdd(&acc[0], sr[0]);
        atomicAdd(&acc[1], sz[0]);
    }
}

// dL/d(o1, o2) of every pair: 2 s (Re, Im) sum_q G_iq conj(Z_jq) / sum |Z|^2,
// times w (the system's loss normalisation).
__global__ void pair_grad_kernel(int64_t P, int nprobe, int64_t n, const int32_t* __restrict__ pi,
                                 const int32_t* __restrict__ pj, const float* __restrict__ scale,
                                 const double2* __restrict__ G, const double2* __restrict__ Z,
                                 const double* __restrict__ acc, double w, float* __restrict__ dO) {
    int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (p >= P) return;
    const int64_t i = pi[p], j = pj[p];
    double re = 0, im = 0;
    for (int q = 0; q < nprobe; ++q) {
        double2 g = G[(size_t)q * n + i], z = Z[(size_t)q * n + j];
        re += g.x * z.x + g.y * z.y;
        im += g.y * z.x - g.x * z.y;
    }
    const double f = 2.0 * w * scale[p] / acc[1];
    dO[2 * p] = (float)(f * re);
    dO[2 * p + 1] = (float)(f * im);
}

// D = D * (1 - H^2) (tanh derivative).
__global__ void tanh_back_kernel(int64_t total, const float* __restrict__ H, float* __restrict__ D) {
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t < total) D[t] *= 1.f - H[t] * H[t];
}

// Column sums (bias gradients): out[c] += sum_r D[r][c].
__global__ void colsum_kernel(int64_t rows, int cols, const float* __restrict__ D, float* __restrict__ out) {
    __shared__ float sh[256];
    const int c = blockIdx.x;
    float s = 0.f;
    for (int64_t r = blockIdx.y * (int64_t)blockDim.x + threadIdx.x; r < rows; r += (int64_t)gridDim.y * blockDim.x)
        s += D[r * cols + c];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(&out[c], sh[0]);
}

__global__ void adam_kernel(int n, float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m1,
                            float* __restrict__ m2, float lr, float b1, float b2, float c1, float c2, float eps) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    float gg = g[t];
    float a = b1 * m1[t] + (1.f - b1) * gg;
    float b = b2 * m2[t] + (1.f - b2) * gg * gg;
    m1[t] = a;
    m2[t] = b;
    w[t] -= lr * (a / c1) / (sqrtf(b / c2) + eps);
}

// Backward through the MLP from dO (P x 2) to the parameter gradients (added to grad).
void mlp_backward(Context& c, const LearnedNet& net, int64_t P, const float* F, const float* H1, const float* H2,
                  const float* dO, float* D2, float* D1, float* grad) {
    const float* wb = net.wbf.as<float>();
    const int split = (int)std::min<int64_t>(256, std::max<int64_t>(1, P / 4096));
    // layer 3
    gemm<1, 0>(c, NO, NH, P, dO, H2, grad + OFF_W3, nullptr, 0, 0, split);
    colsum_kernel<<<dim3(NO, 64), 256, 0, c.stream>>>(P, NO, dO, grad + OFF_B3);
    BEM_CHECK_LAUNCH(&c);
    gemm<0, 0>(c, P, NH, NO, dO, wb + OFF_W3, D2, nullptr, 0, 0);
    tanh_back_kernel<<<(unsigned)((P * NH + 255) / 256), 256, 0, c.stream>>>(P * NH, H2, D2);
    BEM_CHECK_LAUNCH(&c);
    // layer 2
    gemm<1, 0>(c, NH, NH, P, D2, H1, grad + OFF_W2, nullptr, 0, 0, split);
    colsum_kernel<<<dim3(NH, 16), 256, 0, c.stream>>>(P, NH, D2, grad + OFF_B2);
    BEM_CHECK_LAUNCH(&c);
    gemm<0, 0>(c, P, NH, NH, D2, wb + OFF_W2, D1, nullptr, 0, 0);
    tanh_back_kernel<<<(unsigned)((P * NH + 255) / 256), 256, 0, c.stream>>>(P * NH, H1, D1);
    BEM_CHECK_LAUNCH(&c);
    // layer 1
    gemm<1, 0>(c, NH, NF, P, D1, F, grad + OFF_W1, nullptr, 0, 0, split);
    colsum_kernel<<<dim3(NH, 16), 256, 0, c.stream>>>(P, NH, D1, grad + OFF_B1);
    BEM_CHECK_LAUNCH(&c);
}

void LearnedNet::init(Context& c, uint64_t seed) {
    std::vector<float> w(NPARAM, 0.f);
    std::mt19937_64 g(seed);
    auto fill = [&](int off, int fan_out, int fan_in, float gain) {
        std::normal_distribution<float> nd(0.f, gain / std::sqrt((float)fan_in));
        for (int t = 0; t < fan_out * fan_in; ++t) w[(size_t)(off + t)] = nd(g);
    };
    fill(OFF_W1, NH, NF, 1.0f);
    fill(OFF_W2, NH, NH, 1.0f);
    // the output layer starts at zero: an untrained network adds nothing to block-Jacobi
    w_host = w;
    upload(c);
    m1.ensure(sizeof(float) * NPARAM);
    m2.ensure(sizeof(float) * NPARAM);
    BEM_CUDA(cudaMemsetAsync(m1.p, 0, sizeof(float) * NPARAM, c.stream));
    BEM_CUDA(cudaMemsetAsync(m2.p, 0, sizeof(float) * NPARAM, c.stream));
    step = 0;
    ready = true;
}

void LearnedNet::upload(Context& c) {
    w.ensure(sizeof(float) * NPARAM);
    wbf.ensure(sizeof(float) * NPARAM);
    BEM_CUDA(cudaMemcpyAsync(w.p, w_host.data(), sizeof(float) * NPARAM, cudaMemcpyHostToDevice, c.stream));
    refresh(c);
}

void LearnedNet::refresh(Context& c) {
    round_params_kernel<<<(NPARAM + 255) / 256, 256, 0, c.stream>>>(NPARAM, w.as<float>(), wbf.as<float>());
    BEM_CHECK_LAUNCH(&c);
}

int learned_num_params() { return NPARAM; }

// ---------------------------------------------------------------------------
// Preconditioner data of a batch (one body, nsys frequencies).
struct PcData {
    NearPattern pat;  // one body, or the concatenated leaves of several
    DevBuf cl_off, cl_idx, nb_off, nb_d, nb_blk, M;
    DevBuf sys_body, body_leaf0, sys_moff;  // several bodies
    bool multi = false;
    int nc_max = 0;  // leaves of the largest body
    size_t m_total = 0;
    PcDev dev(int use_off) const {
        PcDev d;
        d.cl_off = cl_off.as<int64_t>();
        d.cl_idx = cl_idx.as<int64_t>();
        d.nb_blk = nb_blk.as<int64_t>();
        d.nb_off = nb_off.as<int32_t>();
        d.nb_d = nb_d.as<int32_t>();
        d.M = M.as<float2>();
        d.Mstride = (size_t)pat.entries;
        d.offdiag = use_off;
        d.nc = pat.nc;
        d.sys_body = multi ? sys_body.as<int32_t>() : nullptr;
        d.body_leaf0 = multi ? body_leaf0.as<int32_t>() : nullptr;
        d.sys_moff = multi ? sys_moff.as<size_t>() : nullptr;
        d.sys_off = gated ? sys_off.as<int8_t>() : nullptr;
        return d;
    }
    DevBuf sys_off;
    bool gated = false;
};

static void upload_pattern(Context& c, PcData& d) {
    auto up = [&](DevBuf& b, const void* h, size_t bytes) {
        b.ensure(bytes ? bytes : 16);
        if (bytes) BEM_CUDA(cudaMemcpyAsync(b.p, h, bytes, cudaMemcpyHostToDevice, c.stream));
    };
    up(d.cl_off, d.pat.cl_off.data(), sizeof(int64_t) * d.pat.cl_off.size());
    up(d.cl_idx, d.pat.cl_idx.data(), sizeof(int64_t) * d.pat.cl_idx.size());
    up(d.nb_off, d.pat.nb_off.data(), sizeof(int32_t) * d.pat.nb_off.size());
    up(d.nb_d, d.pat.nb_d.data(), sizeof(int32_t) * d.pat.nb_d.size());
    up(d.nb_blk, d.pat.nb_blk.data(), sizeof(int64_t) * d.pat.nb_blk.size());
}

// Block-Jacobi inverses of every system of a batch into d.M (`sys`: ragged
// batch layout, else uniform with lda / mstride).
static void diag_inverses(Context& c, PcData& d, int nsys, const void* A, bool fp32, int64_t lda, size_t mstride,
                          const GmSys* sys = nullptr) {
    const size_t total = d.multi ? d.m_total : (size_t)d.pat.entries * nsys;
    d.M.ensure(sizeof(float2) * std::max<size_t>(total, 1));
    BEM_CUDA(cudaMemsetAsync(d.M.p, 0, sizeof(float2) * total, c.stream));
    int bmax = 0;
    for (int cc = 0; cc < d.pat.nc; ++cc)
        bmax = std::max(bmax, (int)(d.pat.cl_off[cc + 1] - d.pat.cl_off[cc]));
    size_t smem = sizeof(float2) * (size_t)bmax * 2 * bmax;
    // the attribute is set to the cap for leaf clusters of PC_LEAF points on
    // every call (the same value from every thread; a per-call value could
    // lower it under a concurrent larger launch)
    const int smem_cap = (int)(sizeof(float2) * PC_LEAF * 2 * PC_LEAF);
    require(smem <= (size_t)smem_cap, "block-Jacobi: leaf cluster larger than the leaf size", BEM_ERR_CUDA);
    dim3 grid((unsigned)(d.multi ? d.nc_max : d.pat.nc), (unsigned)nsys);
    if (fp32) {
        BEM_CUDA(cudaFuncSetAttribute(pc_diag_inverse_kernel<float2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      smem_cap));
        pc_diag_inverse_kernel<float2><<<grid, 256, smem, c.stream>>>(static_cast<const float2*>(A), lda, mstride,
                                                                      sys, d.dev(0), d.M.as<float2>());
    } else {
        BEM_CUDA(cudaFuncSetAttribute(pc_diag_inverse_kernel<double2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      smem_cap));
        pc_diag_inverse_kernel<double2><<<grid, 256, smem, c.stream>>>(static_cast<const double2*>(A), lda, mstride,
                                                                       sys, d.dev(0), d.M.as<float2>());
    }
    BEM_CHECK_LAUNCH(&c);
}

// Learned off-diagonal entries of system s (wavenumber k) into d.M.
struct PairBufs {
    DevBuf pi, pj, dst, F, scale, H1, H2, O;
};

// The pattern's pair lists on the device, and the per-pair buffers: the
// features and scales, plus the activations when the network is trained.
static void upload_pairs(Context& c, const NearPattern& pat, PairBufs& b, bool training) {
    const int64_t P = std::max<int64_t>(pat.npairs, 1);
    b.pi.ensure(sizeof(int32_t) * P);
    b.pj.ensure(sizeof(int32_t) * P);
    b.dst.ensure(sizeof(int64_t) * P);
    if (pat.npairs) {
        BEM_CUDA(cudaMemcpyAsync(b.pi.p, pat.pair_i.data(), sizeof(int32_t) * pat.npairs, cudaMemcpyHostToDevice,
                                 c.stream));
        BEM_CUDA(cudaMemcpyAsync(b.pj.p, pat.pair_j.data(), sizeof(int32_t) * pat.npairs, cudaMemcpyHostToDevice,
                                 c.stream));
        BEM_CUDA(cudaMemcpyAsync(b.dst.p, pat.pair_dst.data(), sizeof(int64_t) * pat.npairs, cudaMemcpyHostToDevice,
                                 c.stream));
    }
    b.F.ensure(sizeof(float) * P * NF);
    b.scale.ensure(sizeof(float) * P);
    if (training) {
        b.H1.ensure(sizeof(float) * P * NH);
        b.H2.ensure(sizeof(float) * P * NH);
        b.O.ensure(sizeof(float) * P * NO);
    }
}

// The learned entries of one system: features of its P pairs (pi, pj, dst
// on the device) into F / scale (room for P pairs), then tensor-core
// inference writing s_p (o_1 + i o_2) into the system's blocks Ms.
static void learned_entries(Context& c, const Problem& p, const LearnedNet& net, int64_t P, const int32_t* pi,
                            const int32_t* pj, const int64_t* dst, float* F, float* scale, double k, float2* Ms,
                            bool check) {
    if (P == 0) return;
    pc_features_kernel<<<(unsigned)((P + 255) / 256), 256, 0, c.stream>>>(P, pi, pj, p.geo.npad, p.geo.arr(0), k,
                                                                          F, scale);
    BEM_CHECK_LAUNCH(&c);
    mlp_infer_tc(c, net, P, F, nullptr, dst, scale, Ms, check);
}

struct PcHookData {
    PcData data;
    bool use_off;
};

static void pc_hook(Context& c, GmWorkspace& ws, int mode, void* user) {
    (void)mode;
    PcHookData& h = *static_cast<PcHookData*>(user);
    dim3 grid((unsigned)(h.data.multi ? h.data.nc_max : h.data.pat.nc), (unsigned)ws.bt.nsys);
    pc_apply_gmres_kernel<<<grid, PC_LEAF, 0, c.stream>>>(h.data.dev(h.use_off ? 1 : 0), ws.bt);
    BEM_CHECK_LAUNCH(&c);
}

// Block-Jacobi is the learned form's fallback: for every system the learned
// correction is kept only where it lowers the probe residual
// E ||A M z - z||^2 / ||z||^2 (GATE_PROBES random probes, the same for both)
// below GATE_KEEP times block-Jacobi's.  FP32 operators only (the refined
// form's FP64 operators keep the correction).  Returns the systems kept.
constexpr int GATE_PROBES = 2;
constexpr double GATE_KEEP = 0.95;

// One system of the gate's batch: size, leading dimension, operator offset
// (float2 entries) and the offset of its probe vectors.
struct GateSys {
    int64_t n, lda, aoff, voff;
};

// Y = M_s Z for every system s (blockIdx.z) and probe (blockIdx.y).
__global__ void __launch_bounds__(PC_LEAF) gate_apply_kernel(PcDev pc, const GateSys* __restrict__ gs,
                                                             const double2* __restrict__ Z, double2* __restrict__ Y) {
    const int s = blockIdx.z, q = blockIdx.y;
    const int c = pc_leaf(pc, s, blockIdx.x);
    if (c < 0) return;
    const GateSys g = gs[s];
    const size_t v = (size_t)g.voff + (size_t)q * g.n;
    pc_block_apply(c, pc.cl_off, pc.cl_idx, pc.nb_off, pc.nb_d, pc.nb_blk, pc.M + pc_moff(pc, s), Z + v, Y + v,
                   pc.offdiag);
}

// W = A_s Y and the residual partials |W - Z|^2, |Z|^2 of every system and
// probe in one launch: a thread per row, FP32 arithmetic (the gate compares
// two estimates), the sums accumulated per system.
__global__ void gate_residual_kernel(const float2* __restrict__ A, const GateSys* __restrict__ gs,
                                     const double2* __restrict__ Y, const double2* __restrict__ Z,
                                     double* __restrict__ acc) {
    __shared__ double sr[128], sz[128];
    const int s = blockIdx.z, q = blockIdx.y;
    const GateSys g = gs[s];
    const int64_t i = (int64_t)blockIdx.x * 128 + threadIdx.x;
    double a = 0, b = 0;
    if (i < g.n) {
        const size_t v = (size_t)g.voff + (size_t)q * g.n;
        const float2* As = A + g.aoff + i;
        float ax = 0.f, ay = 0.f;
        for (int64_t j = 0; j < g.n; ++j) {
            const float2 e = As[j * g.lda];
            const double2 y = Y[v + j];
            const float yx = (float)y.x, yy = (float)y.y;
            ax = fmaf(e.x, yx, fmaf(-e.y, yy, ax));
            ay = fmaf(e.x, yy, fmaf(e.y, yx, ay));
        }
        const double2 z = Z[v + i];
        const double rx = (double)ax - z.x, ry = (double)ay - z.y;
        a = rx * rx + ry * ry;
        b = z.x * z.x + z.y * z.y;
    }
    sr[threadIdx.x] = a;
    sz[threadIdx.x] = b;
    __syncthreads();
    for (int o = 64; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            sr[threadIdx.x] += sr[threadIdx.x + o];
            sz[threadIdx.x] += sz[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        atomicAdd(acc + 2 * s, sr[0]);
        atomicAdd(acc + 2 * s + 1, sz[0]);
    }
}

static int learned_gate(Context& c, PcData& d, GmWorkspace& ws, uint64_t seed) {
    const int nsys = ws.bt.nsys;
    if (!ws.fp32) return nsys;
    std::vector<GateSys> gs((size_t)nsys);
    int64_t tot = 0, nmax = 0;
    for (int s = 0; s < nsys; ++s) {
        GateSys& g = gs[(size_t)s];
        g.n = ws.sys_host.empty() ? ws.bt.n : ws.sys_host[(size_t)s].n;
        g.lda = ws.sys_host.empty() ? ws.bt.lda : ws.sys_host[(size_t)s].lda;
        g.aoff = (int64_t)(ws.sys_host.empty() ? (size_t)s * ws.bt.mat_stride : ws.sys_host[(size_t)s].a_off);
        g.voff = tot;
        tot += g.n * GATE_PROBES;
        nmax = std::max(nmax, g.n);
    }
    DevBuf Z, Y, acc, dgs;
    Z.ensure(sizeof(double2) * (size_t)tot);
    Y.ensure(sizeof(double2) * (size_t)tot);
    acc.ensure(sizeof(double) * 4 * (size_t)nsys);
    dgs.ensure(sizeof(GateSys) * (size_t)nsys);
    BEM_CUDA(cudaMemcpyAsync(dgs.p, gs.data(), sizeof(GateSys) * nsys, cudaMemcpyHostToDevice, c.stream));
    BEM_CUDA(cudaMemsetAsync(acc.p, 0, sizeof(double) * 4 * (size_t)nsys, c.stream));
    // the same probes for block-Jacobi (use 0) and the learned form (use 1)
    probes_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, c.stream>>>(tot, seed * 2654435761ull, Z.as<double2>());
    BEM_CHECK_LAUNCH(&c);
    const int nleaf = d.multi ? d.nc_max : d.pat.nc;
    for (int use = 0; use < 2; ++use) {
        gate_apply_kernel<<<dim3((unsigned)nleaf, (unsigned)GATE_PROBES, (unsigned)nsys), PC_LEAF, 0, c.stream>>>(
            d.dev(use), dgs.as<GateSys>(), Z.as<double2>(), Y.as<double2>());
        BEM_CHECK_LAUNCH(&c);
        gate_residual_kernel<<<dim3((unsigned)((nmax + 127) / 128), (unsigned)GATE_PROBES, (unsigned)nsys), 128, 0,
                               c.stream>>>(static_cast<const float2*>(ws.bt.A), dgs.as<GateSys>(), Y.as<double2>(),
                                           Z.as<double2>(), acc.as<double>() + 2 * (size_t)nsys * use);
        BEM_CHECK_LAUNCH(&c);
    }
    std::vector<double> h(4 * (size_t)nsys);
    BEM_CUDA(cudaMemcpyAsync(h.data(), acc.p, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, c.stream));
    c.sync();
    std::vector<int8_t> keep((size_t)nsys);
    int kept = 0;
    for (int s = 0; s < nsys; ++s) {
        const double* u0 = h.data() + 2 * (size_t)s;                  // block-Jacobi
        const double* u1 = h.data() + 2 * ((size_t)nsys + (size_t)s);  // learned
        const double bj = u0[0] / u0[1], ln = u1[0] / u1[1];
        keep[(size_t)s] = (int8_t)(std::isfinite(ln) && ln < GATE_KEEP * bj);
        kept += keep[(size_t)s];
    }
    d.sys_off.ensure(std::max<size_t>((size_t)nsys, 1));
    BEM_CUDA(cudaMemcpyAsync(d.sys_off.p, keep.data(), (size_t)nsys, cudaMemcpyHostToDevice, c.stream));
    c.sync();
    d.gated = true;
    return kept;
}

namespace {
// Wall time of a preconditioner set-up (it ends synchronised) for the
// library's per-stage profile.
struct SetupTimer {
    Context& c;
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    int64_t l0;
    explicit SetupTimer(Context& ctx) : c(ctx), l0(ctx.launches) {}
    ~SetupTimer() {
        if (!c.profiling) return;
        cudaStreamSynchronize(c.stream);
        c.stage_add("precond_setup",
                    std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count(),
                    c.launches - l0, 0);
    }
};
// Wall time of one part of a set-up (synchronised at its end) when profiling.
struct PartTimer {
    Context& c;
    const char* name;
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    PartTimer(Context& ctx, const char* n) : c(ctx), name(n) {}
    ~PartTimer() {
        if (!c.profiling) return;
        cudaStreamSynchronize(c.stream);
        c.stage_add(name, std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count(),
                    0, 0);
    }
};
}  // namespace

bem_precond precond_setup(Context& c, Problem& p, GmWorkspace& ws, bem_precond kind, const double* ks) {
    SetupTimer timer(c);
    if (kind == BEM_PRECOND_LU) {
        lu_precond_setup(c, ws);  // FP64 operators are factored from their FP32 rounding
        return kind;
    }
    require(kind == BEM_PRECOND_BLOCK_JACOBI || kind == BEM_PRECOND_LEARNED, "unknown preconditioner");
    // without a trained or loaded network the learned form falls back to block-Jacobi
    if (kind == BEM_PRECOND_LEARNED && !(c.net && c.net->ready)) kind = BEM_PRECOND_BLOCK_JACOBI;
    auto h = std::make_shared<PcHookData>();
    // block-Jacobi needs the diagonal blocks only
    {
        PartTimer pt(c, "pc_patterns");
        std::vector<NearPattern> pats;
        build_patterns(c, std::vector<const Problem*>{&p}, pats, kind != BEM_PRECOND_LEARNED);
        h->data.pat = std::move(pats[0]);
        upload_pattern(c, h->data);
    }
    const int nsys = ws.bt.nsys;
    {
        PartTimer pt(c, "pc_diag_inverses");
        diag_inverses(c, h->data, nsys, ws.bt.A, ws.fp32, ws.bt.lda, ws.bt.mat_stride, ws.bt.sys);
    }
    h->use_off = false;
    if (kind == BEM_PRECOND_LEARNED) {
        {
            PartTimer pt(c, "pc_learned_entries");
            PairBufs pb;
            upload_pairs(c, h->data.pat, pb, false);
            BEM_CUDA(cudaMemsetAsync(device_err(c), 0, sizeof(int), c.stream));
            for (int s = 0; s < nsys; ++s)
                learned_entries(c, p, *c.net, h->data.pat.npairs, pb.pi.as<int32_t>(), pb.pj.as<int32_t>(),
                                pb.dst.as<int64_t>(), pb.F.as<float>(), pb.scale.as<float>(), ks[s],
                                h->data.M.as<float2>() + (size_t)s * h->data.pat.entries, false);
            h->use_off = true;
            check_device_err(c);
        }
        PartTimer pt(c, "pc_gate");
        learned_gate(c, h->data, ws, 17);
    }
    ws.zb().ensure(sizeof(double2) * gm_q_total(ws));
    ws.bt.Z = ws.zb().as<double2>();
    ws.precond = pc_hook;
    ws.precond_user = h.get();
    ws.precond_keep = h;
    return kind;
}

// Several bodies in one ragged batch: system s belongs to body sys_body[s]
// (wavenumber ks[s]); the bodies' leaf patterns are concatenated and every
// system's blocks are stored back to back.
bem_precond precond_setup_multi(Context& c, const std::vector<Problem*>& bodies, const std::vector<int>& sys_body,
                                GmWorkspace& ws, bem_precond kind, const double* ks) {
    SetupTimer timer(c);
    if (kind == BEM_PRECOND_LU) {
        lu_precond_setup(c, ws);
        return kind;
    }
    require(kind == BEM_PRECOND_BLOCK_JACOBI || kind == BEM_PRECOND_LEARNED, "unknown preconditioner");
    require(!ws.sys_host.empty() && (int)sys_body.size() == ws.bt.nsys, "multi-body preconditioner: bad batch");
    if (kind == BEM_PRECOND_LEARNED && !(c.net && c.net->ready)) kind = BEM_PRECOND_BLOCK_JACOBI;
    const bool learned = kind == BEM_PRECOND_LEARNED;
    auto h = std::make_shared<PcHookData>();
    PcData& d = h->data;
    const int nb = (int)bodies.size(), nsys = ws.bt.nsys;
    std::vector<NearPattern> pats;
    {
        PartTimer pt(c, "pc_patterns");
        build_patterns(c, std::vector<const Problem*>(bodies.begin(), bodies.end()), pats, !learned);
    }
    std::vector<int32_t> leaf0(1, 0);
    NearPattern& P = d.pat;
    P.cl_off.assign(1, 0);
    P.nb_off.assign(1, 0);
    for (int b = 0; b < nb; ++b) {
        const NearPattern& q = pats[(size_t)b];
        const int64_t idx0 = (int64_t)P.cl_idx.size();
        const int32_t nb0 = (int32_t)P.nb_d.size();
        for (int l = 0; l < q.nc; ++l) {
            P.cl_off.push_back(idx0 + q.cl_off[(size_t)l + 1]);
            P.nb_off.push_back(nb0 + q.nb_off[(size_t)l + 1]);
        }
        P.cl_idx.insert(P.cl_idx.end(), q.cl_idx.begin(), q.cl_idx.end());
        for (int32_t x : q.nb_d) P.nb_d.push_back(x + leaf0.back());
        P.nb_blk.insert(P.nb_blk.end(), q.nb_blk.begin(), q.nb_blk.end());
        d.nc_max = std::max(d.nc_max, q.nc);
        leaf0.push_back(leaf0.back() + q.nc);
    }
    P.nc = leaf0.back();
    P.entries = 0;
    std::vector<size_t> moff((size_t)nsys);
    size_t tot = 0;
    for (int s = 0; s < nsys; ++s) {
        moff[(size_t)s] = tot;
        tot += (size_t)pats[(size_t)sys_body[(size_t)s]].entries;
    }
    d.m_total = tot;
    d.multi = true;
    upload_pattern(c, d);
    d.sys_body.ensure(sizeof(int32_t) * nsys);
    d.body_leaf0.ensure(sizeof(int32_t) * leaf0.size());
    d.sys_moff.ensure(sizeof(size_t) * nsys);
    BEM_CUDA(cudaMemcpyAsync(d.sys_body.p, sys_body.data(), sizeof(int32_t) * nsys, cudaMemcpyHostToDevice, c.stream));
    BEM_CUDA(cudaMemcpyAsync(d.body_leaf0.p, leaf0.data(), sizeof(int32_t) * leaf0.size(), cudaMemcpyHostToDevice,
                             c.stream));
    BEM_CUDA(cudaMemcpyAsync(d.sys_moff.p, moff.data(), sizeof(size_t) * nsys, cudaMemcpyHostToDevice, c.stream));
    {
        PartTimer pt(c, "pc_diag_inverses");
        diag_inverses(c, d, nsys, ws.bt.A, ws.fp32, 0, 0, ws.bt.sys);
    }
    h->use_off = false;
    if (learned) {
        PartTimer pt(c, "pc_learned_entries");
        // every body's pair lists on the device at once; the systems then
        // run back to back through one feature / scale buffer (stream
        // order), with no host round trip between them
        std::vector<int64_t> poff((size_t)nb + 1, 0);
        int64_t pmax = 1;
        for (int b = 0; b < nb; ++b) {
            poff[(size_t)b + 1] = poff[(size_t)b] + pats[(size_t)b].npairs;
            pmax = std::max(pmax, pats[(size_t)b].npairs);
        }
        PairBufs pb;
        const int64_t ptot = std::max<int64_t>(poff[(size_t)nb], 1);
        pb.pi.ensure(sizeof(int32_t) * ptot);
        pb.pj.ensure(sizeof(int32_t) * ptot);
        pb.dst.ensure(sizeof(int64_t) * ptot);
        pb.F.ensure(sizeof(float) * pmax * NF);
        pb.scale.ensure(sizeof(float) * pmax);
        for (int b = 0; b < nb; ++b) {
            const NearPattern& q = pats[(size_t)b];
            if (q.npairs == 0) continue;
            const size_t o = (size_t)poff[(size_t)b];
            BEM_CUDA(cudaMemcpyAsync(pb.pi.as<int32_t>() + o, q.pair_i.data(), sizeof(int32_t) * q.npairs,
                                     cudaMemcpyHostToDevice, c.stream));
            BEM_CUDA(cudaMemcpyAsync(pb.pj.as<int32_t>() + o, q.pair_j.data(), sizeof(int32_t) * q.npairs,
                                     cudaMemcpyHostToDevice, c.stream));
            BEM_CUDA(cudaMemcpyAsync(pb.dst.as<int64_t>() + o, q.pair_dst.data(), sizeof(int64_t) * q.npairs,
                                     cudaMemcpyHostToDevice, c.stream));
        }
        BEM_CUDA(cudaMemsetAsync(device_err(c), 0, sizeof(int), c.stream));
        for (int s = 0; s < nsys; ++s) {
            const int b = sys_body[(size_t)s];
            const size_t o = (size_t)poff[(size_t)b];
            learned_entries(c, *bodies[(size_t)b], *c.net, pats[(size_t)b].npairs, pb.pi.as<int32_t>() + o,
                            pb.pj.as<int32_t>() + o, pb.dst.as<int64_t>() + o, pb.F.as<float>(),
                            pb.scale.as<float>(), ks[s], d.M.as<float2>() + moff[(size_t)s], false);
        }
        check_device_err(c);
        h->use_off = true;
    }
    if (learned) {
        PartTimer pt(c, "pc_gate");
        learned_gate(c, d, ws, 17);
    }
    c.sync();
    ws.zb().ensure(sizeof(double2) * gm_q_total(ws));
    ws.bt.Z = ws.zb().as<double2>();
    ws.precond = pc_hook;
    ws.precond_user = h.get();
    ws.precond_keep = h;
    return kind;
}

// ---------------------------------------------------------------------------
// Training on the operators of a set of problems (all their frequencies).
double learned_train(Context& c, std::vector<Problem*>& probs, int steps, int nprobe, double lr, uint64_t seed,
                     std::vector<double>& losses) {
    if (!c.net) c.net = std::make_unique<LearnedNet>();
    if (!c.net->ready) c.net->init(c, seed);
    LearnedNet& net = *c.net;
    struct Sys {
        Problem* p;
        int f;
        double k;
    };
    struct Body {
        Problem* p;
        PcData pc;
        PairBufs pb;
        DevBuf A;
        int64_t lda;
        size_t mstride;
        int nf;
        std::vector<double> ks;
    };
    std::vector<std::unique_ptr<Body>> bodies;
    std::vector<NearPattern> pats;
    build_patterns(c, std::vector<const Problem*>(probs.begin(), probs.end()), pats, false);
    for (Problem* p : probs) {
        auto b = std::make_unique<Body>();
        b->p = p;
        b->pc.pat = std::move(pats[bodies.size()]);
        upload_pattern(c, b->pc);
        upload_pairs(c, b->pc.pat, b->pb, true);
        b->nf = (int)p->freqs.size();
        b->lda = p->geo.npad;
        b->mstride = (size_t)b->lda * p->n;
        b->A.ensure(sizeof(float2) * b->mstride * b->nf);
        std::vector<cd> al(b->nf), be(b->nf), ga(b->nf), de(b->nf);
        int64_t saved = p->ifreq;
        for (int f = 0; f < b->nf; ++f) {
            p->ifreq = f;
            b->ks.push_back(p->wavenumber());
            lhs_factors(*p, al[f], be[f]);
            rhs_factors(*p, ga[f], de[f]);
        }
        p->ifreq = saved;
        DevBuf nrm;
        nrm.ensure(sizeof(double) * b->nf);
        assemble_system_fp32_body(c, *p, b->ks.data(), al.data(), be.data(), ga.data(), de.data(), b->nf,
                                  b->A.as<float2>(), b->lda, b->mstride, nullptr, 0, nrm.as<double>());
        diag_inverses(c, b->pc, b->nf, b->A.p, true, b->lda, b->mstride);
        c.sync();
        bodies.push_back(std::move(b));
    }
    require(!bodies.empty(), "no training problems");
    DevBuf grad, lossacc, D1, D2, dO, Z, Y, W, R, G;
    grad.ensure(sizeof(float) * NPARAM);
    lossacc.ensure(sizeof(double) * 2);
    int64_t pmax = 1, nmax = 1;
    for (auto& b : bodies) {
        pmax = std::max(pmax, b->pc.pat.npairs);
        nmax = std::max(nmax, b->p->n);
    }
    D1.ensure(sizeof(float) * pmax * NH);
    D2.ensure(sizeof(float) * pmax * NH);
    dO.ensure(sizeof(float) * pmax * NO);
    for (DevBuf* v : {&Z, &Y, &W, &R, &G}) v->ensure(sizeof(double2) * (size_t)nmax * nprobe);
    losses.clear();
    // every system's block-Jacobi probe loss (the correction still zero): the
    // training loss of a system is its loss relative to this, so systems of
    // every wavenumber weigh alike (1 = no better than block-Jacobi)
    std::vector<std::vector<double>> lbj(bodies.size());
    for (size_t bi = 0; bi < bodies.size(); ++bi) {
        Body& b = *bodies[bi];
        const int64_t n = b.p->n, tot = n * nprobe;
        for (int f = 0; f < b.nf; ++f) {
            probes_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, c.stream>>>(tot, seed * 104729 + (uint64_t)f,
                                                                                Z.as<double2>());
            BEM_CHECK_LAUNCH(&c);
            pc_apply_probes_kernel<<<dim3((unsigned)b.pc.pat.nc, (unsigned)nprobe), PC_LEAF, 0, c.stream>>>(
                b.pc.dev(1), f, Z.as<double2>(), Y.as<double2>(), n);
            BEM_CHECK_LAUNCH(&c);
            probe_matvec_kernel<<<dim3((unsigned)((n + 127) / 128), (unsigned)nprobe), 128, 0, c.stream>>>(
                n, b.A.as<float2>() + (size_t)f * b.mstride, b.lda, Y.as<double2>(), W.as<double2>(), 0);
            BEM_CHECK_LAUNCH(&c);
            BEM_CUDA(cudaMemsetAsync(lossacc.p, 0, sizeof(double) * 2, c.stream));
            probe_residual_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, c.stream>>>(
                tot, W.as<double2>(), Z.as<double2>(), R.as<double2>(), lossacc.as<double>());
            BEM_CHECK_LAUNCH(&c);
            double la[2];
            BEM_CUDA(cudaMemcpyAsync(la, lossacc.p, sizeof(la), cudaMemcpyDeviceToHost, c.stream));
            c.sync();
            lbj[bi].push_back(std::max(la[0] / la[1], 1e-30));
        }
    }
    int64_t sidx = 0;
    for (int it = 0; it < steps; ++it) {
        const size_t bi = (size_t)((sidx / 1) % bodies.size());
        Body& b = *bodies[bi];
        const int f = (int)((sidx / (int64_t)bodies.size()) % b.nf);
        const double wsys = 1.0 / lbj[bi][(size_t)f];
        ++sidx;
        const int64_t n = b.p->n, P = b.pc.pat.npairs;
        float2* Ms = b.pc.M.as<float2>() + (size_t)f * b.pc.pat.entries;
        const float2* As = b.A.as<float2>() + (size_t)f * b.mstride;
        // forward: features, MLP, learned entries of this system
        if (P > 0) {
            pc_features_kernel<<<(unsigned)((P + 255) / 256), 256, 0, c.stream>>>(
                P, b.pb.pi.as<int32_t>(), b.pb.pj.as<int32_t>(), b.p->geo.npad, b.p->geo.arr(0), b.ks[(size_t)f],
                b.pb.F.as<float>(), b.pb.scale.as<float>());
            BEM_CHECK_LAUNCH(&c);
            mlp_forward(c, net, P, b.pb.F.as<float>(), b.pb.H1.as<float>(), b.pb.H2.as<float>(), b.pb.O.as<float>());
            pc_write_learned_kernel<<<(unsigned)((P + 255) / 256), 256, 0, c.stream>>>(
                P, b.pb.O.as<float>(), b.pb.scale.as<float>(), b.pb.dst.as<int64_t>(), Ms);
            BEM_CHECK_LAUNCH(&c);
        }
        // probe loss: R = A M Z - Z, G = A^H R
        const int64_t tot = n * nprobe;
        probes_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, c.stream>>>(tot, seed * 7919 + (uint64_t)it,
                                                                            Z.as<double2>());
        BEM_CHECK_LAUNCH(&c);
        pc_apply_probes_kernel<<<dim3((unsigned)b.pc.pat.nc, (unsigned)nprobe), PC_LEAF, 0, c.stream>>>(
            b.pc.dev(1), f, Z.as<double2>(), Y.as<double2>(), n);
        BEM_CHECK_LAUNCH(&c);
        probe_matvec_kernel<<<dim3((unsigned)((n + 127) / 128), (unsigned)nprobe), 128, 0, c.stream>>>(
            n, As, b.lda, Y.as<double2>(), W.as<double2>(), 0);
        BEM_CHECK_LAUNCH(&c);
        BEM_CUDA(cudaMemsetAsync(lossacc.p, 0, sizeof(double) * 2, c.stream));
        probe_residual_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, c.stream>>>(
            tot, W.as<double2>(), Z.as<double2>(), R.as<double2>(), lossacc.as<double>());
        BEM_CHECK_LAUNCH(&c);
        probe_matvec_kernel<<<dim3((unsigned)((n * 32 + 127) / 128), (unsigned)nprobe), 128, 0, c.stream>>>(
            n, As, b.lda, R.as<double2>(), G.as<double2>(), 1);
        BEM_CHECK_LAUNCH(&c);
        double la[2];
        BEM_CUDA(cudaMemcpyAsync(la, lossacc.p, sizeof(la), cudaMemcpyDeviceToHost, c.stream));
        // backward and Adam
        BEM_CUDA(cudaMemsetAsync(grad.p, 0, sizeof(float) * NPARAM, c.stream));
        if (P > 0) {
            pair_grad_kernel<<<(unsigned)((P + 255) / 256), 256, 0, c.stream>>>(
                P, nprobe, n, b.pb.pi.as<int32_t>(), b.pb.pj.as<int32_t>(), b.pb.scale.as<float>(), G.as<double2>(),
                Z.as<double2>(), lossacc.as<double>(), wsys, dO.as<float>());
            BEM_CHECK_LAUNCH(&c);
            mlp_backward(c, net, P, b.pb.F.as<float>(), b.pb.H1.as<float>(), b.pb.H2.as<float>(), dO.as<float>(),
                         D2.as<float>(), D1.as<float>(), grad.as<float>());
        }
        net.step += 1;
        const float b1 = 0.9f, b2 = 0.999f;
        const float c1 = 1.f - std::pow(b1, (float)net.step), c2 = 1.f - std::pow(b2, (float)net.step);
        adam_kernel<<<(NPARAM + 255) / 256, 256, 0, c.stream>>>(NPARAM, net.w.as<float>(), grad.as<float>(),
                                                                 net.m1.as<float>(), net.m2.as<float>(), (float)lr, b1,
                                                                 b2, c1, c2, 1e-8f);
        BEM_CHECK_LAUNCH(&c);
        net.refresh(c);
        c.sync();
        losses.push_back(wsys * la[0] / la[1]);
    }
    net.w_host.resize(NPARAM);
    BEM_CUDA(cudaMemcpyAsync(net.w_host.data(), net.w.p, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost, c.stream));
    c.sync();
    return losses.empty() ? 0.0 : losses.back();
}

// Tensor-core inference on caller features (host arrays).
void learned_mlp_infer(Context& c, int64_t P, const float* hF, float* hO) {
    require(c.net && c.net->ready, "no network loaded");
    DevBuf F, O;
    F.ensure(sizeof(float) * P * NF);
    O.ensure(sizeof(float) * P * NO);
    BEM_CUDA(cudaMemcpyAsync(F.p, hF, sizeof(float) * P * NF, cudaMemcpyHostToDevice, c.stream));
    mlp_infer_tc(c, *c.net, P, F.as<float>(), O.as<float>(), nullptr, nullptr, nullptr);
    BEM_CUDA(cudaMemcpyAsync(hO, O.p, sizeof(float) * P * NO, cudaMemcpyDeviceToHost, c.stream));
    c.sync();
}

// MLP forward (and backward for given output gradients) on caller features:
// exposes the network kernels for checking against a CPU restatement.
void learned_mlp_eval(Context& c, int64_t P, const float* hF, const float* hdO, float* hO, float* hgrad) {
    require(c.net && c.net->ready, "no network loaded");
    DevBuf F, H1, H2, O, dO, D1, D2, grad;
    F.ensure(sizeof(float) * P * NF);
    H1.ensure(sizeof(float) * P * NH);
    H2.ensure(sizeof(float) * P * NH);
    O.ensure(sizeof(float) * P * NO);
    BEM_CUDA(cudaMemcpyAsync(F.p, hF, sizeof(float) * P * NF, cudaMemcpyHostToDevice, c.stream));
    mlp_forward(c, *c.net, P, F.as<float>(), H1.as<float>(), H2.as<float>(), O.as<float>());
    if (hO) BEM_CUDA(cudaMemcpyAsync(hO, O.p, sizeof(float) * P * NO, cudaMemcpyDeviceToHost, c.stream));
    if (hdO && hgrad) {
        dO.ensure(sizeof(float) * P * NO);
        D1.ensure(sizeof(float) * P * NH);
        D2.ensure(sizeof(float) * P * NH);
        grad.ensure(sizeof(float) * NPARAM);
        BEM_CUDA(cudaMemcpyAsync(dO.p, hdO, sizeof(float) * P * NO, cudaMemcpyHostToDevice, c.stream));
        BEM_CUDA(cudaMemsetAsync(grad.p, 0, sizeof(float) * NPARAM, c.stream));
        mlp_backward(c, *c.net, P, F.as<float>(), H1.as<float>(), H2.as<float>(), dO.as<float>(), D2.as<float>(),
                     D1.as<float>(), grad.as<float>());
        BEM_CUDA(cudaMemcpyAsync(hgrad, grad.p, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost, c.stream));
    }
    c.sync();
}

}  // namespace bem
