// Preconditioners for the batched GMRES.
#include "common.cuh"
#include "precond.cuh"

namespace bem {

void precond_setup(Context& c, Problem& p, GmWorkspace& ws, bem_precond kind, const double* ks) {
    (void)c; (void)p; (void)ws; (void)ks;
    throw Error(BEM_ERR_BAD_INPUT, "preconditioner " + std::to_string((int)kind) + " is not available");
}

}  // namespace bem
