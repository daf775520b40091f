// Mixed form, single-precision assembly and field evaluation.
//
// A_s = alpha_s H_s + beta_s G_s is assembled for several frequencies s of one
// body in one pass: the geometry-only terms of a pair (separation, direction
// cosines) are evaluated once and reused for every frequency.  Coordinates are
// float-float (hi + lo) so the separation r is accurate to ~1e-14 relative;
// the phase k r is formed in float-float and reduced modulo pi/2 (Cody-Waite
// with an exact FMA product), and sin/cos on |x| <= pi/4 use Taylor
// polynomials (truncation < 2e-9).  The singular self term stays FP64.  The
// same kernel accumulates the squared Frobenius norm of every A_s (needed by
// the GMRES stopping test) so the operators are never re-read for it.
#include "common.cuh"
#include "complex.cuh"
#include "ff.cuh"
#include "kernels.cuh"
#include "tma.cuh"

namespace bem {

// Per-frequency constants.  Those that scale every off-diagonal entry carry a
// lo part: the diagonal (self term) is formed in FP64, so a rounded constant
// would perturb the off-diagonal part of the operator coherently, an error the
// solve amplifies by the condition number (unlike independent roundings).
struct Sys32 {
    float kh, kl;             // wavenumber hi + lo
    float bih, bil;           // 1/k hi + lo (Burton-Miller) or 0
    float k2;                 // k^2
    float2 alpha, beta;       // LHS factors, hi
    float2 alpha_l, beta_l;   // LHS factors, lo
    float2 gamma, delta;      // RHS factors
    double kd, gdiag_im;
    int alpha_one, beta_zero; // alpha = 1 and beta = 0 exactly (most boundary conditions)
};

// The frequency-dependent constants of one system.
static void set_sys32(Sys32& S, double k, bool bm, cd alpha, cd beta) {
    S.kh = (float)k;
    S.kl = (float)(k - (double)S.kh);
    S.kd = k;
    S.k2 = (float)(k * k);
    const double bi = bm ? 1.0 / k : 0.0;
    S.bih = (float)bi;
    S.bil = (float)(bi - (double)S.bih);
    S.gdiag_im = bm ? 0.5 * (1.0 / k) : 0.0;
    S.alpha = make_float2((float)alpha.re, (float)alpha.im);
    S.beta = make_float2((float)beta.re, (float)beta.im);
    S.alpha_l = make_float2((float)(alpha.re - (double)S.alpha.x), (float)(alpha.im - (double)S.alpha.y));
    S.beta_l = make_float2((float)(beta.re - (double)S.beta.x), (float)(beta.im - (double)S.beta.y));
    S.alpha_one = alpha.re == 1.0 && alpha.im == 0.0;
    S.beta_zero = beta.re == 0.0 && beta.im == 0.0;
}

// c * x for a float-float constant (ch + cl) and a float x: rounded once.
__device__ __forceinline__ float ffmul(float ch, float cl, float x) { return fmaf(ch, x, cl * x); }
// (ch + cl) * z for float-float complex constant parts and a complex z.
__device__ __forceinline__ float2 ffcmul(float2 ch, float2 cl, float2 z) {
    return make_float2(fmaf(ch.x, z.x, fmaf(-ch.y, z.y, cl.x * z.x - cl.y * z.y)),
                       fmaf(ch.x, z.y, fmaf(ch.y, z.x, cl.x * z.y + cl.y * z.x)));
}
constexpr int MAX_SYS32 = 16;
struct Asm32Params {
    int nsys, bm;
    double hdiag;
    float P1, P2, P3, two_over_pi;
    Sys32 s[MAX_SYS32];
};

struct TileGeo32 {
    float cxh[TILE], cxl[TILE], cyh[TILE], cyl[TILE], czh[TILE], czl[TILE], cex[TILE], cey[TILE], cez[TILE], cwa[TILE];
    float cexl[TILE], ceyl[TILE], cezl[TILE], cwal[TILE];
    float rxh[TILE], rxl[TILE], ryh[TILE], ryl[TILE], rzh[TILE], rzl[TILE], rex[TILE], rey[TILE], rez[TILE];
    float rexl[TILE], reyl[TILE], rezl[TILE];
};

// a - b as float-float (hi, lo) given float-float inputs.
__device__ __forceinline__ void ff_diff(float ah, float al, float bh, float bl, float& h, float& l) {
    float s = ah - bh;
    float bb = s - ah;
    float e = (ah - (s - bb)) - (bh + bb);
    h = s;
    l = e + (al - bl);
}

__device__ __forceinline__ void two_sum32(float a, float b, float& s, float& e) {
    s = a + b;
    float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// sin and cos on |x| <= pi/4 + eps from their Taylor series (terms through
// x^9 and x^10), Horner form.
__device__ __forceinline__ void poly_sincos(float x, float& s, float& c) {
    const float x2 = x * x;
    float ps = fmaf(x2, 2.75573192e-6f, -1.98412698e-4f);   // 1/9!, -1/7!
    ps = fmaf(x2, ps, 8.33333333e-3f);                       // 1/5!
    ps = fmaf(x2, ps, -1.66666667e-1f);                      // -1/3!
    s = fmaf(x * x2, ps, x);
    float pc = fmaf(x2, -2.75573192e-7f, 2.48015873e-5f);   // -1/10!, 1/8!
    pc = fmaf(x2, pc, -1.38888889e-3f);                      // -1/6!
    pc = fmaf(x2, pc, 4.16666667e-2f);                       // 1/4!
    pc = fmaf(x2, pc, -0.5f);                                // -1/2!
    c = fmaf(x2, pc, 1.0f);
}

// e^{i k r} with k = kh + kl and r = rh + rl (float-float).
__device__ __forceinline__ void phase32(float kh, float kl, float rh, float rl, const Asm32Params& prm, float& c0,
                                        float& s0) {
    float p = kh * rh;
    float pe = fmaf(kh, rh, -p) + (kh * rl + kl * rh);
    float nq = rintf(p * prm.two_over_pi);
    float tt = nq * prm.P2;
    float te = fmaf(nq, prm.P2, -tt);
    float red = ((fmaf(-nq, prm.P1, p) - tt) + ((pe - te) - nq * prm.P3));
    float sn, cs;
    poly_sincos(red, sn, cs);
    int quad = ((int)nq) & 3;
    c0 = cs;
    s0 = sn;
    if (quad == 1) { c0 = -sn; s0 = cs; }
    else if (quad == 2) { c0 = -cs; s0 = -sn; }
    else if (quad == 3) { c0 = sn; s0 = -cs; }
}

// r = |a - b| for float-float points: returns the separation (float-float),
// r hi/lo and 1/r.
struct Sep32 {
    float dxh, dxl, dyh, dyl, dzh, dzl, rh, rl, inv;
};

// d . n for a float-float separation d and a float-float unit normal n,
// rounded once (exact products and sums of the hi parts, first-order terms of
// the lo parts).  Between neighbouring elements d is nearly tangent and the
// plain FP32 dot product loses most of its digits to cancellation.
__device__ __forceinline__ float dot_ff(const Sep32& d, float nxh, float nxl, float nyh, float nyl, float nzh,
                                        float nzl) {
    const float p1 = d.dxh * nxh, p2 = d.dyh * nyh, p3 = d.dzh * nzh;
    const float e1 = fmaf(d.dxh, nxh, -p1), e2 = fmaf(d.dyh, nyh, -p2), e3 = fmaf(d.dzh, nzh, -p3);
    float s1, t1, s2, t2;
    two_sum32(p1, p2, s1, t1);
    two_sum32(s1, p3, s2, t2);
    const float lo = (t1 + t2) + (e1 + e2 + e3) + (fmaf(d.dxh, nxl, d.dxl * nxh) + fmaf(d.dyh, nyl, d.dyl * nyh) +
                                                    fmaf(d.dzh, nzl, d.dzl * nzh));
    return s2 + lo;
}
__device__ __forceinline__ Sep32 separation32(float axh, float axl, float ayh, float ayl, float azh, float azl,
                                              float bxh, float bxl, float byh, float byl, float bzh, float bzl) {
    float dxh, dxl, dyh, dyl, dzh, dzl;
    ff_diff(axh, axl, bxh, bxl, dxh, dxl);
    ff_diff(ayh, ayl, byh, byl, dyh, dyl);
    ff_diff(azh, azl, bzh, bzl, dzh, dzl);
    float px = dxh * dxh, py = dyh * dyh, pz = dzh * dzh;
    float ex = fmaf(dxh, dxh, -px), ey = fmaf(dyh, dyh, -py), ez = fmaf(dzh, dzh, -pz);
    float s1, e1, s2, e2;
    two_sum32(px, py, s1, e1);
    two_sum32(s1, pz, s2, e2);
    float r2l = (e1 + e2) + (ex + ey + ez) + 2.0f * (dxh * dxl + dyh * dyl + dzh * dzl);
    Sep32 o;
    o.rh = sqrtf(s2);
    o.rl = (fmaf(-o.rh, o.rh, s2) + r2l) * (0.5f / o.rh);
    // 1/r from r rounded once: s2 holds the squares of the hi parts only, off
    // by ~1e-6 between neighbouring elements (the near-field terms carry 1/r
    // up to the third power)
    o.inv = 1.0f / (o.rh + o.rl);
    o.dxh = dxh;
    o.dxl = dxl;
    o.dyh = dyh;
    o.dyl = dyl;
    o.dzh = dzh;
    o.dzl = dzl;
    return o;
}

struct Asm32Smem {
    TileGeo32 t;
    uint64_t bar;
    float red[ASM_THREADS / 32][MAX_SYS32];
};

// One 64 x 64 tile (row tile ti, column tile tj) of every system of a body;
// the squared Frobenius norm partial of system s goes to
// norm_part[s * norm_stride + tile_index].
template <int WITH_RHS>
__device__ __forceinline__ void assemble32_tile(int64_t n, int64_t npad, const float* __restrict__ g32,
                                                const double* __restrict__ geo, const Asm32Params& prm,
                                                float2* __restrict__ A, int64_t ld, size_t mat_stride,
                                                double2* __restrict__ part, size_t part_stride,
                                                double* __restrict__ norm_part, size_t norm_stride,
                                                size_t tile_index, int ti, int tj, int* __restrict__ err,
                                                Asm32Smem& sm) {
    TileGeo32& t = sm.t;
    uint64_t& bar = sm.bar;
    auto& red = sm.red;
    const int64_t I0 = (int64_t)ti * TILE, J0 = (int64_t)tj * TILE;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    const uint32_t B = TILE * sizeof(float);
    if (threadIdx.x == 0) {
        mbar_arrive_expect_tx(&bar, 26 * B);
        float* cdst[14] = {t.cxh,  t.cxl, t.cyh,  t.cyl,  t.czh,  t.czl,  t.cex,
                           t.cey,  t.cez, t.cwa,  t.cexl, t.ceyl, t.cezl, t.cwal};
        for (int a = 0; a < 14; ++a) bulk_g2s(cdst[a], g32 + a * npad + J0, B, &bar);
        float* rdst[13] = {t.rxh, t.rxl, t.ryh, t.ryl, t.rzh, t.rzl, t.rex, t.rey, t.rez, nullptr, t.rexl, t.reyl, t.rezl};
        for (int a = 0; a < 13; ++a)
            if (rdst[a]) bulk_g2s(rdst[a], g32 + a * npad + I0, B, &bar);
    }
    if (!mbar_wait_bounded(&bar, 0)) {
        if (threadIdx.x == 0) atomicOr(err, DEVERR_MBAR_TIMEOUT);
        mbar_wait_bounded(&bar, 0);
        return;
    }
    const int tx = threadIdx.x & (TILE - 1), ty = threadIdx.x >> 6;
    const int64_t i = I0 + tx;
    const float yxh = t.rxh[tx], yxl = t.rxl[tx], yyh = t.ryh[tx], yyl = t.ryl[tx], yzh = t.rzh[tx],
                yzl = t.rzl[tx];
    const float eyx = t.rex[tx], eyy = t.rey[tx], eyz = t.rez[tx];
    const float eyxl = t.rexl[tx], eyyl = t.reyl[tx], eyzl = t.rezl[tx];
    float nrm[MAX_SYS32];
    float2 acc[MAX_SYS32];
#pragma unroll
    for (int s = 0; s < MAX_SYS32; ++s) {
        nrm[s] = 0.f;
        acc[s] = make_float2(0.f, 0.f);
    }
#pragma unroll 1
    for (int c = 0; c < TILE / 4; ++c) {
        const int jj = ty + 4 * c;
        const int64_t j = J0 + jj;
        const bool store = i < n && j < n;
        if (i == j) {
            if (!store) continue;
            double area = geo[GAREA * npad + j], wt = geo[GWT * npad + j];
#pragma unroll
            for (int s = 0; s < MAX_SYS32; ++s) {
                if (s >= prm.nsys) break;
                z2 g, h;
                self_term64(area, wt, prm.bm, prm.bm ? 1.0 / prm.s[s].kd : 0.0, prm.hdiag, prm.s[s].gdiag_im, g, h);
                z2 al = make_double2(prm.s[s].alpha.x, prm.s[s].alpha.y);
                z2 be = make_double2(prm.s[s].beta.x, prm.s[s].beta.y);
                z2 a = cmul(al, h);
                cfma(a, be, g);
                float2 af = make_float2((float)a.x, (float)a.y);
                A[s * mat_stride + j * ld + i] = af;
                nrm[s] += af.x * af.x + af.y * af.y;
                if (WITH_RHS) {
                    z2 ga = make_double2(prm.s[s].gamma.x, prm.s[s].gamma.y);
                    z2 de = make_double2(prm.s[s].delta.x, prm.s[s].delta.y);
                    z2 r = cmul(ga, h);
                    cfma(r, de, g);
                    acc[s].x += (float)r.x;
                    acc[s].y += (float)r.y;
                }
            }
            continue;
        }
        const Sep32 sp = separation32(t.cxh[jj], t.cxl[jj], t.cyh[jj], t.cyl[jj], t.czh[jj], t.czl[jj], yxh, yxl, yyh,
                                      yyl, yzh, yzl);
        const float inv = sp.inv;
        const float rdoty = dot_ff(sp, eyx, eyxl, eyy, eyyl, eyz, eyzl) * inv;
        const float rdotx = dot_ff(sp, t.cex[jj], t.cexl[jj], t.cey[jj], t.ceyl[jj], t.cez[jj], t.cezl[jj]) * inv;
        const float nxy = eyx * t.cex[jj] + eyy * t.cey[jj] + eyz * t.cez[jj];
        const float q = fmaf(inv, t.cwa[jj], inv * t.cwal[jj]);  // wt * area / (4 pi r)
#pragma unroll
        for (int s = 0; s < MAX_SYS32; ++s) {
            if (s >= prm.nsys) break;
            const Sys32& S = prm.s[s];
            float c0, s0;
            phase32(S.kh, S.kl, sp.rh, sp.rl, prm, c0, s0);
            float2 g = make_float2(c0 * q, s0 * q);  // g * wt * area
            // g f1 with f1 = i k - 1/r
            float2 gf1 = make_float2(-fmaf(g.x, inv, ffmul(S.kh, S.kl, g.y)), fmaf(-g.y, inv, ffmul(S.kh, S.kl, g.x)));
            float2 h = fscale(gf1, -rdoty);
            if (prm.bm) {
                float2 dg = fscale(gf1, rdotx);
                float2 t1 = make_float2(inv * nxy, -ffmul(S.kh, S.kl, nxy));  // (-f1) * nxy
                float2 t2 = fscale(make_float2(S.k2 * sp.rh - 3.0f * inv, 3.0f * S.kh), rdotx * rdoty);
                float2 dh = fmul(fscale(g, inv), make_float2(t1.x - t2.x, t1.y - t2.y));
                g = make_float2(g.x - ffmul(S.bih, S.bil, dg.y), g.y + ffmul(S.bih, S.bil, dg.x));
                h = make_float2(h.x - ffmul(S.bih, S.bil, dh.y), h.y + ffmul(S.bih, S.bil, dh.x));
            }
            if (store) {
                // alpha h + beta g (uniform branches: alpha is 1 for every
                // boundary condition but pressure, beta is 0 for velocity)
                float2 af = S.alpha_one ? h : ffcmul(S.alpha, S.alpha_l, h);
                if (!S.beta_zero) {
                    const float2 b2 = ffcmul(S.beta, S.beta_l, g);
                    af = make_float2(af.x + b2.x, af.y + b2.y);
                }
                A[s * mat_stride + j * ld + i] = af;
                nrm[s] += af.x * af.x + af.y * af.y;
                if (WITH_RHS) {
                    float2 r1 = fmul(S.gamma, h), r2 = fmul(S.delta, g);
                    acc[s].x += r1.x + r2.x;
                    acc[s].y += r1.y + r2.y;
                }
            }
        }
    }
    // squared Frobenius norms: warp shuffle, then one partial per CTA
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int s = 0; s < MAX_SYS32; ++s) {
        if (s >= prm.nsys) break;
        float v = nrm[s];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp][s] = v;
    }
    __syncthreads();
    if (threadIdx.x < prm.nsys) {
        double sum = 0;
        for (int w = 0; w < ASM_THREADS / 32; ++w) sum += red[w][threadIdx.x];
        norm_part[(size_t)threadIdx.x * norm_stride + tile_index] = sum;
    }
    if (WITH_RHS) {
        __shared__ float2 rred[ASM_THREADS];
#pragma unroll
        for (int s = 0; s < MAX_SYS32; ++s) {
            if (s >= prm.nsys) break;
            __syncthreads();
            rred[threadIdx.x] = acc[s];
            __syncthreads();
            if (ty == 0 && i < n) {
                double sx = 0, sy = 0;
                for (int q2 = 0; q2 < 4; ++q2) {
                    sx += rred[tx + TILE * q2].x;
                    sy += rred[tx + TILE * q2].y;
                }
                part[s * part_stride + (int64_t)tj * npad + i] = make_double2(sx, sy);
            }
        }
    }
}

// MINB: CTAs per SM the register allocation must allow (tuned per size:
// more CTAs hide latency, fewer registers per thread cost spills and ILP).
template <int WITH_RHS, int MINB = 3>
__global__ void __launch_bounds__(ASM_THREADS, MINB) assemble32_kernel(
    int64_t n, int64_t npad, const float* __restrict__ g32, const double* __restrict__ geo, Asm32Params prm,
    float2* __restrict__ A, int64_t ld, size_t mat_stride, double2* __restrict__ part, size_t part_stride,
    double* __restrict__ norm_part, int* __restrict__ err) {
    __shared__ __align__(128) Asm32Smem sm;
    assemble32_tile<WITH_RHS>(n, npad, g32, geo, prm, A, ld, mat_stride, part, part_stride, norm_part,
                              (size_t)gridDim.x * gridDim.y, (size_t)blockIdx.y * gridDim.x + blockIdx.x,
                              (int)blockIdx.y, (int)blockIdx.x, err, sm);
}

// Several bodies (each with its own frequencies) in one launch: a flattened
// grid over every body's tiles, the body found by bisection on tile0 and its
// parameters staged in shared memory.
struct Body32 {
    int64_t n, npad;
    const float* g32;
    const double* geo;
    float2* A;          // system s of the body at A + s * mat_stride
    int64_t ld;
    size_t mat_stride;
    double* norm_part;  // nsys x ntiles^2 partials
    int64_t tile0;
    int ntiles, pad;
};

__global__ void __launch_bounds__(ASM_THREADS, 3) assemble32_multi_kernel(const Body32* __restrict__ bodies,
                                                                      int nbodies,
                                                                      const Asm32Params* __restrict__ prms,
                                                                      int* __restrict__ err) {
    __shared__ __align__(128) Asm32Smem sm;
    __shared__ __align__(16) Asm32Params prm;
    const int64_t t = blockIdx.x;
    int lo = 0, hi = nbodies - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (bodies[mid].tile0 <= t) lo = mid;
        else hi = mid - 1;
    }
    const Body32 B = bodies[lo];
    {
        const int* src = reinterpret_cast<const int*>(prms + lo);
        int* dst = reinterpret_cast<int*>(&prm);
        for (int w = threadIdx.x; w < (int)(sizeof(Asm32Params) / sizeof(int)); w += ASM_THREADS) dst[w] = src[w];
    }
    __syncthreads();
    const int64_t local = t - B.tile0;
    const int ti = (int)(local / B.ntiles), tj = (int)(local % B.ntiles);
    assemble32_tile<0>(B.n, B.npad, B.g32, B.geo, prm, B.A, B.ld, B.mat_stride, nullptr, 0, B.norm_part,
                       (size_t)B.ntiles * B.ntiles, (size_t)local, ti, tj, err, sm);
}

__global__ void finish_norm_kernel(const double* __restrict__ part, int64_t nparts, double* __restrict__ out) {
    __shared__ double sh[256];
    const int s = blockIdx.x;
    double v = 0;
    for (int64_t t = threadIdx.x; t < nparts; t += blockDim.x) v += part[(size_t)s * nparts + t];
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[s] = sqrt(sh[0]);
}

// out[s] = sqrt(sum of the nparts partials of system s).
void finish_norms(Context& ctx, const double* part, int64_t nparts, int nsys, double* out) {
    finish_norm_kernel<<<nsys, 256, 0, ctx.stream>>>(part, nparts, out);
    BEM_CHECK_LAUNCH(&ctx);
}


// ---------------------------------------------------------------------------
// Split FP64 operators in float-float (refined form and first-kind systems).
// The entry formula of the FP64 assembly (influence_matrix.rs:170-230: the
// Burton-Miller combination alpha H + beta G) evaluated in float-float on the
// FP32 pipe: separation, 1/r, direction cosines and phase in float-float,
// e^{ik r} by ff_cossin (once per pair and the recurrence e^{ik_s r} =
// e^{ik_0 r} e^{i dk r}^s for evenly spaced wavenumbers, as the FP64 kernel
// does), the singular self term in FP64.  Each entry is stored as its float
// pair: the high plane is the operator rounded to FP32, the low plane (plane
// float2 further on) the remainder, ~2^-44 relative to the FP64 value.
struct SysFF {
    ff k, k2, bi;        // wavenumber, k^2, 1/k (Burton-Miller) or 0
    cff alpha, beta;     // LHS factors
    int alpha_one, beta_zero;
    double kd, beta_im, gdiag_im;
    double2 alpha_d, beta_d;
};
constexpr int MAX_SYSFF = 16;
struct AsmFFParams {
    int nsys, bm, recur, pad;
    double hdiag;
    ff k0, dk;           // recurrence: k_s = k0 + s dk
    SysFF s[MAX_SYSFF];
};

__device__ __forceinline__ ff ffd(float h, float l) { return ff{h, l}; }

template <bool SPLIT>
__global__ void __launch_bounds__(ASM_THREADS, 2) assemble_ff_kernel(int64_t n, int64_t npad,
                                                                    const float* __restrict__ g32,
                                                                    const double* __restrict__ geo, AsmFFParams prm,
                                                                    float2* __restrict__ A, int64_t ld, size_t stride,
                                                                    size_t plane, double* __restrict__ norm_part,
                                                                    int* __restrict__ err) {
    __shared__ __align__(128) Asm32Smem sm;
    TileGeo32& t = sm.t;
    const int64_t I0 = (int64_t)blockIdx.y * TILE, J0 = (int64_t)blockIdx.x * TILE;
    if (threadIdx.x == 0) {
        mbar_init(&sm.bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    const uint32_t B = TILE * sizeof(float);
    if (threadIdx.x == 0) {
        mbar_arrive_expect_tx(&sm.bar, 26 * B);
        float* cdst[14] = {t.cxh,  t.cxl, t.cyh,  t.cyl,  t.czh,  t.czl,  t.cex,
                           t.cey,  t.cez, t.cwa,  t.cexl, t.ceyl, t.cezl, t.cwal};
        for (int a = 0; a < 14; ++a) bulk_g2s(cdst[a], g32 + a * npad + J0, B, &sm.bar);
        float* rdst[13] = {t.rxh, t.rxl, t.ryh, t.ryl, t.rzh, t.rzl, t.rex, t.rey, t.rez, nullptr, t.rexl, t.reyl, t.rezl};
        for (int a = 0; a < 13; ++a)
            if (rdst[a]) bulk_g2s(rdst[a], g32 + a * npad + I0, B, &sm.bar);
    }
    if (!mbar_wait_bounded(&sm.bar, 0)) {
        if (threadIdx.x == 0) atomicOr(err, DEVERR_MBAR_TIMEOUT);
        mbar_wait_bounded(&sm.bar, 0);
        return;
    }
    const int tx = threadIdx.x & (TILE - 1), ty = threadIdx.x >> 6;
    const int64_t i = I0 + tx;
    const float yxh = t.rxh[tx], yxl = t.rxl[tx], yyh = t.ryh[tx], yyl = t.ryl[tx], yzh = t.rzh[tx],
                yzl = t.rzl[tx];
    const ff eyx = ffd(t.rex[tx], t.rexl[tx]), eyy = ffd(t.rey[tx], t.reyl[tx]), eyz = ffd(t.rez[tx], t.rezl[tx]);
    float nrm[MAX_SYSFF];
#pragma unroll
    for (int s = 0; s < MAX_SYSFF; ++s) nrm[s] = 0.f;
#pragma unroll 1
    for (int c = 0; c < TILE / 4; ++c) {
        const int jj = ty + 4 * c;
        const int64_t j = J0 + jj;
        if (i >= n || j >= n) continue;
        const size_t o = (size_t)(j * ld + i);
        if (i == j) {
            const double area = geo[GAREA * npad + j], wt = geo[GWT * npad + j];
#pragma unroll 1
            for (int s = 0; s < prm.nsys; ++s) {
                z2 g, h;
                self_term64(area, wt, prm.bm, prm.s[s].beta_im, prm.hdiag, prm.s[s].gdiag_im, g, h);
                z2 a = cmul(prm.s[s].alpha_d, h);
                cfma(a, prm.s[s].beta_d, g);
                const float hx = __double2float_rn(a.x), hy = __double2float_rn(a.y);
                A[s * stride + o] = make_float2(hx, hy);
                if (SPLIT)
                    A[s * stride + o + plane] =
                        make_float2(__double2float_rn(a.x - (double)hx), __double2float_rn(a.y - (double)hy));
                nrm[s] += hx * hx + hy * hy;
            }
            continue;
        }
        // separation d = x_j - y_i, r, 1/r, direction cosines (float-float)
        const ff dx = ff_sub(t.cxh[jj], t.cxl[jj], yxh, yxl);
        const ff dy = ff_sub(t.cyh[jj], t.cyl[jj], yyh, yyl);
        const ff dz = ff_sub(t.czh[jj], t.czl[jj], yzh, yzl);
        const ff r = ff_sqrt(dx * dx + dy * dy + dz * dz);
        const ff inv = ff_recip(r);
        const ff exj = ffd(t.cex[jj], t.cexl[jj]), eyj = ffd(t.cey[jj], t.ceyl[jj]), ezj = ffd(t.cez[jj], t.cezl[jj]);
        const ff rdoty = (dx * eyx + dy * eyy + dz * eyz) * inv;
        const ff rdotx = (dx * exj + dy * eyj + dz * ezj) * inv;
        const ff nxy = eyx * exj + eyy * eyj + eyz * ezj;
        const ff q = inv * ffd(t.cwa[jj], t.cwal[jj]);  // wt area / (4 pi r)
        cff e, step;
        if (prm.recur) {
            ff_cossin(prm.k0 * r, e.re, e.im);
            ff_cossin(prm.dk * r, step.re, step.im);
        }
        const ff rr = rdotx * rdoty;
#pragma unroll 1
        for (int s = 0; s < prm.nsys; ++s) {
            const SysFF& S = prm.s[s];
            if (prm.recur) {
                if (s) e = e * step;
            } else {
                ff_cossin(S.k * r, e.re, e.im);
            }
            cff g = e * q;
            // g f1 with f1 = i k - 1/r
            const cff gf1 = times_i(g, S.k) - g * inv;
            cff h = gf1 * (-rdoty);
            if (prm.bm) {
                const cff dg = gf1 * rdotx;
                const cff t1 = cff{inv * nxy, -(S.k * nxy)};                  // (-f1) nxy
                const cff t2 = cff{(S.k2 * r - 3.0f * inv) * rr, (3.0f * S.k) * rr};
                const cff dh = (g * inv) * (t1 - t2);
                g = g + times_i(dg, S.bi);
                h = h + times_i(dh, S.bi);
            }
            cff a = S.alpha_one ? h : S.alpha * h;
            if (!S.beta_zero) a = a + S.beta * g;
            A[s * stride + o] = make_float2(a.re.h, a.im.h);
            if (SPLIT) A[s * stride + o + plane] = make_float2(a.re.l, a.im.l);
            nrm[s] += a.re.h * a.re.h + a.im.h * a.im.h;
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int s = 0; s < MAX_SYSFF; ++s) {
        if (s >= prm.nsys) break;
        float v = nrm[s];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) sm.red[warp][s] = v;
    }
    __syncthreads();
    if (threadIdx.x < prm.nsys) {
        double sum = 0;
        for (int w = 0; w < ASM_THREADS / 32; ++w) sum += sm.red[w][threadIdx.x];
        norm_part[(size_t)threadIdx.x * gridDim.x * gridDim.y + (size_t)blockIdx.y * gridDim.x + blockIdx.x] = sum;
    }
}

static ff host_ff(double v) {
    const float h = (float)v;
    return ff{h, (float)(v - (double)h)};
}

void assemble_system_split(Context& ctx, const Problem& p, const double* ks, const cd* alphas, const cd* betas,
                           int nsys, float2* A, int64_t ld, size_t plane, double* norms, bool remainder) {
    require(plane == (size_t)ld * p.n, "split assembly: planes must be ld * n entries");
    int* err = device_err(ctx);
    BEM_CUDA(cudaMemsetAsync(err, 0, sizeof(int), ctx.stream));
    const int ntiles = (int)(p.geo.npad / TILE);
    const int64_t nparts = (int64_t)ntiles * ntiles;
    ctx.w_norm.ensure(sizeof(double) * (size_t)nparts * MAX_SYSFF);
    const KParams kp = kparams(p);
    for (int s0 = 0; s0 < nsys; s0 += MAX_SYSFF) {
        AsmFFParams prm{};
        prm.nsys = std::min(MAX_SYSFF, nsys - s0);
        prm.bm = kp.bm;
        prm.hdiag = kp.hdiag;
        double kmax = 0;
        for (int s = 0; s < prm.nsys; ++s) {
            const double k = ks[s0 + s];
            SysFF& S = prm.s[s];
            S.k = host_ff(k);
            S.k2 = host_ff(k * k);
            S.bi = host_ff(kp.bm ? 1.0 / k : 0.0);
            const cd al = alphas[s0 + s], be = betas[s0 + s];
            S.alpha = cff{host_ff(al.re), host_ff(al.im)};
            S.beta = cff{host_ff(be.re), host_ff(be.im)};
            S.alpha_one = al.re == 1.0 && al.im == 0.0;
            S.beta_zero = be.re == 0.0 && be.im == 0.0;
            S.kd = k;
            S.beta_im = kp.bm ? 1.0 / k : 0.0;
            S.gdiag_im = kp.bm ? 0.5 * (1.0 / k) : 0.0;
            S.alpha_d = make_double2(al.re, al.im);
            S.beta_d = make_double2(be.re, be.im);
            kmax = std::max(kmax, std::fabs(k));
        }
        // evenly spaced wavenumbers: the recurrence (the FP64 kernel's rule)
        const double k0 = ks[s0];
        const double dk = prm.nsys > 1 ? (ks[s0 + prm.nsys - 1] - ks[s0]) / (prm.nsys - 1) : 0.0;
        prm.recur = prm.nsys > 1;
        for (int s = 0; s < prm.nsys && prm.recur; ++s)
            if (std::fabs(ks[s0 + s] - (k0 + s * dk)) > 1e-13 * kmax) prm.recur = 0;
        prm.k0 = host_ff(k0);
        prm.dk = host_ff(dk);
        dim3 grid((unsigned)ntiles, (unsigned)ntiles);
        // split: systems 2 plane apart, the remainder a plane after each;
        // rounded only: systems a plane apart
        const size_t stride = remainder ? 2 * plane : plane;
        if (remainder)
            assemble_ff_kernel<true><<<grid, ASM_THREADS, 0, ctx.stream>>>(
                p.n, p.geo.npad, p.geo.arr32(0), p.geo.arr(0), prm, A + (size_t)s0 * stride, ld, stride, plane,
                ctx.w_norm.as<double>(), err);
        else
            assemble_ff_kernel<false><<<grid, ASM_THREADS, 0, ctx.stream>>>(
                p.n, p.geo.npad, p.geo.arr32(0), p.geo.arr(0), prm, A + (size_t)s0 * stride, ld, stride, plane,
                ctx.w_norm.as<double>(), err);
        BEM_CHECK_LAUNCH(&ctx);
        finish_norms(ctx, ctx.w_norm.as<double>(), nparts, prm.nsys, norms + s0);
    }
    check_device_err(ctx);
}

void assemble_system_fp32_body(Context& ctx, const Problem& p, const double* ks, const cd* alphas, const cd* betas,
                               const cd* gammas, const cd* deltas, int nsys, float2* A, int64_t ld, size_t mat_stride,
                               double2* rowsum, size_t vec_stride, double* norms) {
    int* err = device_err(ctx);
    BEM_CUDA(cudaMemsetAsync(err, 0, sizeof(int), ctx.stream));
    const float P1 = 1.5703125f;  // 201/128: n * P1 exact for n < 2^16
    const double rem1 = PI_D / 2 - (double)P1;
    const float P2 = (float)rem1;
    const float P3 = (float)(rem1 - (double)P2);
    const int ntiles = (int)(p.geo.npad / TILE);
    const int64_t nparts = (int64_t)ntiles * ntiles;
    DevBuf& nbuf = ctx.w_norm;
    nbuf.ensure(sizeof(double) * (size_t)nparts * MAX_SYS32);
    for (int s0 = 0; s0 < nsys; s0 += MAX_SYS32) {
        Asm32Params prm;
        prm.nsys = std::min(MAX_SYS32, nsys - s0);
        prm.bm = p.in.method_type == 1;
        prm.hdiag = p.in.problem_type == 1 ? -0.5 : 0.0;
        prm.P1 = P1;
        prm.P2 = P2;
        prm.P3 = P3;
        prm.two_over_pi = (float)(2.0 / PI_D);
        for (int s = 0; s < prm.nsys; ++s) {
            double k = ks[s0 + s];
            Sys32& S = prm.s[s];
            set_sys32(S, k, prm.bm, alphas[s0 + s], betas[s0 + s]);
            S.gamma = make_float2((float)gammas[s0 + s].re, (float)gammas[s0 + s].im);
            S.delta = make_float2((float)deltas[s0 + s].re, (float)deltas[s0 + s].im);
        }
        dim3 grid((unsigned)ntiles, (unsigned)ntiles);
        float2* As = A + (size_t)s0 * mat_stride;
        double* np_ = nbuf.as<double>();
        if (rowsum) {
            size_t pstride = (size_t)ntiles * p.geo.npad;
            ctx.w_part.ensure(sizeof(double2) * pstride * prm.nsys);
            double2* part = ctx.w_part.as<double2>();
            assemble32_kernel<1><<<grid, ASM_THREADS, 0, ctx.stream>>>(p.n, p.geo.npad, p.geo.arr32(0), p.geo.arr(0),
                                                                       prm, As, ld, mat_stride, part, pstride, np_,
                                                                       err);
            BEM_CHECK_LAUNCH(&ctx);
            for (int s = 0; s < prm.nsys; ++s)
                launch_reduce_parts(ctx, p.n, p.geo.npad, ntiles, part + s * pstride,
                                    rowsum + (size_t)(s0 + s) * vec_stride);
        } else {
            const int minb = ctx.tuning.pick("assemble32", "min_ctas", p.n, nsys, 3);
            if (minb == 2)
                assemble32_kernel<0, 2><<<grid, ASM_THREADS, 0, ctx.stream>>>(
                    p.n, p.geo.npad, p.geo.arr32(0), p.geo.arr(0), prm, As, ld, mat_stride, nullptr, 0, np_, err);
            else if (minb == 4)
                assemble32_kernel<0, 4><<<grid, ASM_THREADS, 0, ctx.stream>>>(
                    p.n, p.geo.npad, p.geo.arr32(0), p.geo.arr(0), prm, As, ld, mat_stride, nullptr, 0, np_, err);
            else
                assemble32_kernel<0, 3><<<grid, ASM_THREADS, 0, ctx.stream>>>(
                    p.n, p.geo.npad, p.geo.arr32(0), p.geo.arr(0), prm, As, ld, mat_stride, nullptr, 0, np_, err);
            BEM_CHECK_LAUNCH(&ctx);
        }
        if (norms) {
            finish_norm_kernel<<<prm.nsys, 256, 0, ctx.stream>>>(np_, nparts, norms + s0);
            BEM_CHECK_LAUNCH(&ctx);
        }
    }
    check_device_err(ctx);
}

// Norm of system g from its partials part[off[g] .. off[g] + cnt[g]).
__global__ void finish_norm_multi_kernel(const double* __restrict__ part, const int64_t* __restrict__ off,
                                         const int64_t* __restrict__ cnt, double* __restrict__ out) {
    __shared__ double sh[256];
    const int g = blockIdx.x;
    double v = 0;
    for (int64_t t = threadIdx.x; t < cnt[g]; t += blockDim.x) v += part[off[g] + t];
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[g] = sqrt(sh[0]);
}

static void fill_params(const Problem& p, const double* ks, const cd* alphas, const cd* betas, const cd* gammas,
                        const cd* deltas, int nsys, Asm32Params& prm) {
    const float P1 = 1.5703125f;  // 201/128: n * P1 exact for n < 2^16
    const double rem1 = PI_D / 2 - (double)P1;
    prm = Asm32Params{};
    prm.nsys = nsys;
    prm.bm = p.in.method_type == 1;
    prm.hdiag = p.in.problem_type == 1 ? -0.5 : 0.0;
    prm.P1 = P1;
    prm.P2 = (float)rem1;
    prm.P3 = (float)(rem1 - (double)prm.P2);
    prm.two_over_pi = (float)(2.0 / PI_D);
    for (int s = 0; s < nsys; ++s) {
        const double k = ks[s];
        Sys32& S = prm.s[s];
        set_sys32(S, k, prm.bm, alphas[s], betas[s]);
        if (gammas) S.gamma = make_float2((float)gammas[s].re, (float)gammas[s].im);
        if (deltas) S.delta = make_float2((float)deltas[s].re, (float)deltas[s].im);
    }
}

void assemble_fp32_multi(Context& ctx, const std::vector<BodyAsm32>& bodies, double* norms) {
    if (bodies.empty()) return;
    // split bodies with more than MAX_SYS32 systems into entries of <= MAX_SYS32
    std::vector<Body32> ent;
    std::vector<Asm32Params> prms;
    std::vector<int64_t> off, cnt;
    int64_t tiles = 0, parts = 0;
    for (const BodyAsm32& b : bodies) {
        const Problem& p = *b.p;
        const int ntiles = (int)(p.geo.npad / TILE);
        for (int s0 = 0; s0 < b.nsys; s0 += MAX_SYS32) {
            const int ns = std::min(MAX_SYS32, b.nsys - s0);
            Body32 e{};
            e.n = p.n;
            e.npad = p.geo.npad;
            e.g32 = p.geo.arr32(0);
            e.geo = p.geo.arr(0);
            e.A = b.A + (size_t)s0 * b.mat_stride;
            e.ld = b.ld;
            e.mat_stride = b.mat_stride;
            e.norm_part = reinterpret_cast<double*>(parts);  // offset for now
            e.tile0 = tiles;
            e.ntiles = ntiles;
            Asm32Params prm;
            fill_params(p, b.ks + s0, b.alphas + s0, b.betas + s0, nullptr, nullptr, ns, prm);
            for (int s = 0; s < ns; ++s) {
                off.push_back(parts + (int64_t)s * ntiles * ntiles);
                cnt.push_back((int64_t)ntiles * ntiles);
            }
            parts += (int64_t)ns * ntiles * ntiles;
            tiles += (int64_t)ntiles * ntiles;
            ent.push_back(e);
            prms.push_back(prm);
        }
    }
    const size_t nent = ent.size(), nsys = off.size();
    const size_t b_ent = sizeof(Body32) * nent, b_prm = sizeof(Asm32Params) * nent, b_idx = sizeof(int64_t) * nsys;
    DevBuf& nbuf = ctx.w_norm;
    nbuf.ensure(sizeof(double) * (size_t)parts);
    for (Body32& e : ent) e.norm_part = nbuf.as<double>() + reinterpret_cast<int64_t>(e.norm_part);
    DevBuf& meta = ctx.w_small;
    const size_t o_prm = (b_ent + 255) / 256 * 256, o_off = o_prm + (b_prm + 255) / 256 * 256,
                 o_cnt = o_off + (b_idx + 255) / 256 * 256;
    meta.ensure(o_cnt + b_idx);
    char* mb = meta.as<char>();
    BEM_CUDA(cudaMemcpyAsync(mb, ent.data(), b_ent, cudaMemcpyHostToDevice, ctx.stream));
    BEM_CUDA(cudaMemcpyAsync(mb + o_prm, prms.data(), b_prm, cudaMemcpyHostToDevice, ctx.stream));
    BEM_CUDA(cudaMemcpyAsync(mb + o_off, off.data(), b_idx, cudaMemcpyHostToDevice, ctx.stream));
    BEM_CUDA(cudaMemcpyAsync(mb + o_cnt, cnt.data(), b_idx, cudaMemcpyHostToDevice, ctx.stream));
    int* err = device_err(ctx);
    BEM_CUDA(cudaMemsetAsync(err, 0, sizeof(int), ctx.stream));
    require(tiles < (int64_t)INT32_MAX, "multi-body assembly: too many tiles");
    assemble32_multi_kernel<<<(unsigned)tiles, ASM_THREADS, 0, ctx.stream>>>(
        reinterpret_cast<const Body32*>(mb), (int)nent, reinterpret_cast<const Asm32Params*>(mb + o_prm), err);
    BEM_CHECK_LAUNCH(&ctx);
    if (norms) {
        finish_norm_multi_kernel<<<(unsigned)nsys, 256, 0, ctx.stream>>>(
            nbuf.as<double>(), reinterpret_cast<const int64_t*>(mb + o_off), reinterpret_cast<const int64_t*>(mb + o_cnt),
            norms);
        BEM_CHECK_LAUNCH(&ctx);
    }
    check_device_err(ctx);  // synchronises: the host metadata above may be released after return
}

// ---------------------------------------------------------------------------
// Field points for all frequencies in one launch (influence_matrix.rs:101-127
// + solve.rs:173-185 without storing M and L): one CTA per (field point,
// frequency), single-precision kernel evaluation with the float-float phase,
// per-thread sums folded into FP64, fixed-order block reduction.
constexpr int F32_THREADS = 256;
__global__ void __launch_bounds__(F32_THREADS) field32_kernel(
    int64_t nfp, int64_t fpad, const float* __restrict__ fp32, int64_t n, int64_t npad, const float* __restrict__ g32,
    Asm32Params prm, const double2* __restrict__ phi, const double2* __restrict__ vn, int64_t vstride,
    const double2* __restrict__ inc, double2* __restrict__ out) {
    __shared__ double shx[F32_THREADS], shy[F32_THREADS];
    const int64_t i = blockIdx.x;
    const int f = blockIdx.y;
    const Sys32& S = prm.s[f];
    const float pxh = fp32[i], pxl = fp32[fpad + i], pyh = fp32[2 * fpad + i], pyl = fp32[3 * fpad + i],
                pzh = fp32[4 * fpad + i], pzl = fp32[5 * fpad + i];
    const double2* ph = phi + (size_t)f * vstride;
    const double2* vv = vn + (size_t)f * vstride;
    double ax = 0, ay = 0;
    float bx = 0, by = 0;
    int cnt = 0;
    for (int64_t j = threadIdx.x; j < n; j += F32_THREADS) {
        const Sep32 sp = separation32(pxh, pxl, pyh, pyl, pzh, pzl, g32[FXH * npad + j], g32[FXL * npad + j],
                                      g32[FYH * npad + j], g32[FYL * npad + j], g32[FZH * npad + j],
                                      g32[FZL * npad + j]);
        // r = x - y with x the field point, y the element: e_r . n_y
        const float rdoty =
            dot_ff(sp, g32[FEX * npad + j], g32[FEXL * npad + j], g32[FEY * npad + j], g32[FEYL * npad + j],
                   g32[FEZ * npad + j], g32[FEZL * npad + j]) * sp.inv;
        const float q = fmaf(sp.inv, g32[FWA * npad + j], sp.inv * g32[FWAL * npad + j]);  // wt * area / (4 pi r)
        float c0, s0;
        phase32(S.kh, S.kl, sp.rh, sp.rl, prm, c0, s0);
        float2 g = make_float2(c0 * q, s0 * q);
        float2 h = fscale(fmul(g, make_float2(-sp.inv, S.kh)), -rdoty);
        const double2 pj = ph[j], vj = vv[j];
        const float2 pf = make_float2((float)pj.x, (float)pj.y), vf = make_float2((float)vj.x, (float)vj.y);
        const float2 t1 = fmul(h, pf), t2 = fmul(g, vf);
        bx += t2.x - t1.x;
        by += t2.y - t1.y;
        if (++cnt == 8) {
            ax += bx;
            ay += by;
            bx = by = 0;
            cnt = 0;
        }
    }
    shx[threadIdx.x] = ax + bx;
    shy[threadIdx.x] = ay + by;
    __syncthreads();
    for (int o = F32_THREADS / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            shx[threadIdx.x] += shx[threadIdx.x + o];
            shy[threadIdx.x] += shy[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double2 r = make_double2(shx[0], shy[0]);
        if (inc) r = cadd(r, inc[(size_t)f * nfp + i]);
        out[(size_t)f * nfp + i] = r;
    }
}

void evaluate_field32_batch(Context& ctx, const Problem& p, const double* ks, int nsys, const double2* phi,
                            const double2* vn, int64_t vstride, const double2* inc, double2* out) {
    if (p.nfp == 0) return;
    const float P1 = 1.5703125f;
    const double rem1 = PI_D / 2 - (double)P1;
    for (int s0 = 0; s0 < nsys; s0 += MAX_SYS32) {
        Asm32Params prm;
        prm.nsys = std::min(MAX_SYS32, nsys - s0);
        prm.bm = 0;
        prm.hdiag = 0;
        prm.P1 = P1;
        prm.P2 = (float)rem1;
        prm.P3 = (float)(rem1 - (double)prm.P2);
        prm.two_over_pi = (float)(2.0 / PI_D);
        for (int s = 0; s < prm.nsys; ++s) {
            double k = ks[s0 + s];
            prm.s[s].kh = (float)k;
            prm.s[s].kl = (float)(k - (double)prm.s[s].kh);
            prm.s[s].kd = k;
        }
        dim3 grid((unsigned)p.nfp, (unsigned)prm.nsys);
        field32_kernel<<<grid, F32_THREADS, 0, ctx.stream>>>(
            p.nfp, p.nfp_pad, p.d_fp32.as<float>(), p.n, p.geo.npad, p.geo.arr32(0), prm, phi + (size_t)s0 * vstride,
            vn + (size_t)s0 * vstride, vstride, inc ? inc + (size_t)s0 * p.nfp : nullptr, out + (size_t)s0 * p.nfp);
        BEM_CHECK_LAUNCH(&ctx);
    }
}

}  // namespace bem
