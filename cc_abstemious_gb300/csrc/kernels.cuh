// Device helpers shared by the assembly translation units.
#pragma once
#include "common.cuh"
#include "complex.cuh"

namespace bem {

constexpr int TILE = 64;
constexpr int ASM_THREADS = 256;
constexpr double PI_D = 3.14159265358979323846;

// influence_matrix.rs:42-50: static flat-disc self term (k independent), scaled
// by wt*area, plus the hdiag / gdiag diagonal of preprocess.rs:60-74.
__device__ __forceinline__ void self_term64(double area, double wt, int bm, double beta_im, double hdiag,
                                            double gdiag_im, z2& g, z2& h) {
    double b = sqrt(area / PI_D);
    double g0 = 1.0 / (2.0 * PI_D * b);
    double h0im = bm ? beta_im * (-1.0 / (2.0 * PI_D * (b * b * b))) : 0.0;
    g = make_double2(g0 * wt * area, 0.0);
    h = make_double2(0.0, h0im * wt * area);
    h.x += hdiag;
    g.y += gdiag_im;
}

int* device_err(Context& ctx);
void finish_norms(Context& ctx, const double* part, int64_t nparts, int nsys, double* out);
void check_device_err(Context& ctx);
void launch_reduce_parts(Context& ctx, int64_t n, int64_t npad, int ntiles, const double2* part, double2* out);

}  // namespace bem
