// Hierarchical matrices (h_matrix.rs, aca.rs, cluster.rs, block.rs).
#include "common.cuh"
#include "hmatrix.cuh"

namespace bem {

void solve_surface_hmatrix(Context& c, const Problem& p, const double2* d_rhs_inc, double2* d_phi, double2* d_vn,
                           bem_solve_report* rep) {
    (void)c; (void)p; (void)d_rhs_inc; (void)d_phi; (void)d_vn; (void)rep;
    throw Error(BEM_ERR_BAD_INPUT, "Hierarchical solver not built yet");
}

}  // namespace bem

extern "C" {
BEM_API bem_status bem_hmatrix_build(bem_ctx*, const bem_problem*, bem_side, bem_hmatrix** out) {
    if (out) *out = nullptr;
    return BEM_ERR_BAD_INPUT;
}
BEM_API void bem_hmatrix_destroy(bem_hmatrix*) {}
BEM_API bem_status bem_hmatrix_gemv(bem_ctx*, const bem_hmatrix*, bem_cplx, const bem_cplx*, bem_cplx, bem_cplx*) {
    return BEM_ERR_BAD_INPUT;
}
BEM_API double bem_hmatrix_norm(const bem_hmatrix*) { return 0.0; }
BEM_API bem_status bem_hmatrix_stats(const bem_hmatrix*, int64_t*) { return BEM_ERR_BAD_INPUT; }
BEM_API bem_status bem_hmatrix_to_full(bem_ctx*, const bem_hmatrix*, bem_cplx*, int64_t) { return BEM_ERR_BAD_INPUT; }
}
