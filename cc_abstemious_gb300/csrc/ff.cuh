// Float-float ("double-float") arithmetic on the FP32 pipe: a value is the
// unevaluated sum h + l of two floats with |l| <= ulp(h) / 2, about 48
// significant bits.  The error-free transformations are Knuth's two-sum and
// the FMA two-product; addition, multiplication, reciprocal and square root
// follow the double-double algorithms of Dekker (1971) and of Hida, Li and
// Bailey (QD library, 2001) carried over to float pairs.  Sine and cosine
// reduce the argument modulo pi/2 with pi/2 split into three floats
// (Cody-Waite, products exact through FMA) and sum their Taylor series.
#pragma once

#include <cuda_runtime.h>

namespace bem {

struct ff {
    float h, l;
};
struct cff {
    ff re, im;
};

__device__ __forceinline__ ff ffv(float h, float l = 0.f) { return ff{h, l}; }

// s + e = a + b exactly, given |a| >= |b| (or a == 0)
__device__ __forceinline__ ff quick_two_sum(float a, float b) {
    const float s = a + b;
    return ff{s, b - (s - a)};
}
// s + e = a + b exactly
__device__ __forceinline__ ff two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    return ff{s, (a - (s - bb)) + (b - bb)};
}
// p + e = a * b exactly
__device__ __forceinline__ ff two_prod(float a, float b) {
    const float p = a * b;
    return ff{p, fmaf(a, b, -p)};
}

__device__ __forceinline__ ff operator-(ff a) { return ff{-a.h, -a.l}; }
// the "sloppy" sum: relative error ~2^-47 of |a| + |b|
__device__ __forceinline__ ff operator+(ff a, ff b) {
    ff s = two_sum(a.h, b.h);
    return quick_two_sum(s.h, s.l + (a.l + b.l));
}
__device__ __forceinline__ ff operator-(ff a, ff b) { return a + (-b); }
__device__ __forceinline__ ff operator+(ff a, float b) {
    ff s = two_sum(a.h, b);
    return quick_two_sum(s.h, s.l + a.l);
}
__device__ __forceinline__ ff operator*(ff a, ff b) {
    const float p = a.h * b.h;
    float e = fmaf(a.h, b.h, -p);
    e = fmaf(a.h, b.l, fmaf(a.l, b.h, e));
    return quick_two_sum(p, e);
}
__device__ __forceinline__ ff operator*(ff a, float b) {
    const float p = a.h * b;
    const float e = fmaf(a.l, b, fmaf(a.h, b, -p));
    return quick_two_sum(p, e);
}
__device__ __forceinline__ ff operator*(float b, ff a) { return a * b; }

// 1 / b: the float reciprocal refined by one Newton step in float-float.
__device__ __forceinline__ ff ff_recip(ff b) {
    const float y = 1.0f / b.h;
    const ff by = b * y;                       // ~1
    const float r = (1.0f - by.h) - by.l;      // 1 - b y, the first difference exact
    return quick_two_sum(y, y * r);
}
// sqrt(a), a > 0: the float root refined by one Newton step.
__device__ __forceinline__ ff ff_sqrt(ff a) {
    const float s = sqrtf(a.h);
    const float r = fmaf(-s, s, a.h) + a.l;    // a - s^2, the FMA part exact
    return quick_two_sum(s, r * (0.5f / s));
}
// a - b for float-float a and b given as float pairs.
__device__ __forceinline__ ff ff_sub(float ah, float al, float bh, float bl) {
    ff s = two_sum(ah, -bh);
    return quick_two_sum(s.h, s.l + (al - bl));
}

__device__ __forceinline__ cff operator+(cff a, cff b) { return cff{a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ cff operator-(cff a, cff b) { return cff{a.re - b.re, a.im - b.im}; }
__device__ __forceinline__ cff operator*(cff a, cff b) {
    return cff{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
__device__ __forceinline__ cff operator*(cff a, ff s) { return cff{a.re * s, a.im * s}; }
// i * b * z = (-b z.im, b z.re)
__device__ __forceinline__ cff times_i(cff z, ff b) { return cff{-(b * z.im), b * z.re}; }

// cos and sin of a float-float argument 0 <= x < ~1e6 to ~2^-46 relative.
// Reduction: x = n pi/2 + t with pi/2 = P1 + P2 + P3 (the three float
// roundings of pi/2 in turn, remainder ~1e-23) and n P1, n P2 formed exactly;
// then the Taylor series of sin and cos on |t| <= pi/4 (truncated after t^17
// and t^18, below 1e-19): the terms from t^11 and t^10 on in float, the rest
// in float-float, Horner form.
__device__ __forceinline__ void ff_cossin(ff x, ff& c, ff& s) {
    const float P1 = 0x1.921fb6p+0f, P2 = -0x1.777a5cp-25f, P3 = -0x1.ee59dap-50f;
    const float TWO_OVER_PI = 0x1.45f306p-1f;
    const float nf = rintf(x.h * TWO_OVER_PI);
    ff t = x - two_prod(nf, P1);
    t = t - two_prod(nf, P2);
    t = t + (-nf * P3);
    const ff t2 = t * t;
    const float u = t2.h;
    // sin t = t + t^3 (S1 + t^2 (S2 + t^2 (S3 + t^2 (S4 + t^2 tail)))), S_k = (-1)^k / (2k+1)!
    const float ts = fmaf(fmaf(fmaf(0x1.952c78p-49f, u, -0x1.ae7f3ep-41f), u, 0x1.612462p-33f), u, -0x1.ae6456p-26f);
    ff ps = ffv(0x1.71de3ap-19f, 0x1.55b1ccp-45f) + t2 * ts;
    ps = ffv(-0x1.a01a02p-13f, 0x1.7f97fap-39f) + t2 * ps;
    ps = ffv(0x1.111112p-7f, -0x1.dddddep-32f) + t2 * ps;
    ps = ffv(-0x1.555556p-3f, 0x1.555556p-28f) + t2 * ps;
    const ff sn = t + (t * t2) * ps;
    // cos t = 1 + t^2 (C1 + t^2 (C2 + t^2 (C3 + t^2 (C4 + t^2 tail)))), C_k = (-1)^k / (2k)!
    const float tc = fmaf(fmaf(fmaf(fmaf(-0x1.682786p-53f, u, 0x1.ae7f3ep-45f), u, -0x1.93974ap-37f), u,
                               0x1.1eed8ep-29f), u, -0x1.27e4fcp-22f);
    ff pc = ffv(0x1.a01a02p-16f, -0x1.7f97fap-42f) + t2 * tc;
    pc = ffv(-0x1.6c16c2p-10f, 0x1.27d27ep-35f) + t2 * pc;
    pc = ffv(0x1.555556p-5f, -0x1.555556p-30f) + t2 * pc;
    pc = ffv(-0.5f) + t2 * pc;
    const ff cs = ffv(1.0f) + t2 * pc;
    switch (((int)nf) & 3) {
        case 0: c = cs; s = sn; break;
        case 1: c = -sn; s = cs; break;
        case 2: c = -cs; s = -sn; break;
        default: c = sn; s = -cs; break;
    }
}

}  // namespace bem
