// Mixed-precision batched form and FP64-LU error reference.
#pragma once
#include "common.cuh"

namespace bem {

// fp64_operator: the refined form (operators at FP64 accuracy, split);
// rounded: FP32 operators rounded once from their float-float values instead
// of the single-precision assembly (about half its error, ~4x its cost).
void run_mixed(Context& c, Problem& p, bem_precond precond, bem_cplx* scattered, bem_cplx* incident,
               bem_solve_report* reports, bool check_vs_lu, bool fp64_operator = false, bool rounded = false);
// Several bodies: every frequency of every body in one ragged batch (chunks
// of at most budget_bytes of operators; 0: a share of the free memory).
void run_mixed_batch(Context& c, const std::vector<Problem*>& probs, bem_precond precond,
                     bem_cplx* const* scattered, bem_cplx* const* incident, bem_solve_report* const* reports,
                     bool check_vs_lu, size_t budget_bytes);
// ||x - x_LU64|| / ||x_LU64|| for the unknown solved at the problem's current
// frequency (phi for velocity/impedance conditions, vn for pressure).
double lu_reference_error(Context& c, const Problem& p, const double* phi_host, const double* vn_host);

// shared helpers (api.cu)
cd impedance_factor(const Problem& p);
void unpack_solution(Context& c, const Problem& p, const double2* x, double2* phi, double2* vn);
// The same for several systems (problem p at frequency ifreq) in one launch.
struct UnpackItem {
    const Problem* p;
    int64_t ifreq;
    const double2* x;
    double2 *phi, *vn;
};
void unpack_batch(Context& c, const std::vector<UnpackItem>& items);
void launch_rhs_combine(Context& c, int64_t n, double s, const double2* inc, cd bc, const double2* rowsum,
                        double2* out);
void solve_surface_dense_fp64(Context& c, const Problem& p, const double2* d_rhs_inc, double2* d_phi,
                              double2* d_vn, bem_solve_report* rep, double2* d_A_keep, bool reuse_lu = false);

}  // namespace bem
