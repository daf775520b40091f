// Complex arithmetic on double2 / float2 with num-complex's textbook formulas.
#pragma once
#include <cuda_runtime.h>

namespace bem {

typedef double2 z2;
typedef float2 c2;

__host__ __device__ __forceinline__ z2 cadd(z2 a, z2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ z2 csub(z2 a, z2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ z2 cmul(z2 a, z2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ z2 cscale(z2 a, double s) { return make_double2(a.x * s, a.y * s); }
__host__ __device__ __forceinline__ z2 cconj(z2 a) { return make_double2(a.x, -a.y); }
__host__ __device__ __forceinline__ z2 cneg(z2 a) { return make_double2(-a.x, -a.y); }
__host__ __device__ __forceinline__ double cnorm2(z2 a) { return a.x * a.x + a.y * a.y; }
__host__ __device__ __forceinline__ double cabs_(z2 a) { return hypot(a.x, a.y); }
// (a + ib)/(c + id) = ((ac + bd) + i(bc - ad)) / (c^2 + d^2)
__host__ __device__ __forceinline__ z2 cdiv(z2 a, z2 b) {
    double d = b.x * b.x + b.y * b.y;
    return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}
// a += b * c
__host__ __device__ __forceinline__ void cfma(z2& a, z2 b, z2 c) {
    a.x = fma(b.x, c.x, fma(-b.y, c.y, a.x));
    a.y = fma(b.x, c.y, fma(b.y, c.x, a.y));
}

__host__ __device__ __forceinline__ c2 fadd(c2 a, c2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ c2 fmul(c2 a, c2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ c2 fscale(c2 a, float s) { return make_float2(a.x * s, a.y * s); }

}  // namespace bem
