// Hierarchical matrices: cluster / block trees, ACA and the H-matrix mat-vec.
#pragma once
#include "common.cuh"

namespace bem {

struct HMatrixDev;

void solve_surface_hmatrix(Context& c, const Problem& p, const double2* d_rhs_inc, double2* d_phi, double2* d_vn,
                           bem_solve_report* rep);

}  // namespace bem
