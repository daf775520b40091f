// Preconditioners for the batched GMRES (block-Jacobi and learned).
#pragma once
#include "common.cuh"
#include "gmres.cuh"

namespace bem {

void precond_setup(Context& c, Problem& p, GmWorkspace& ws, bem_precond kind, const double* ks);

}  // namespace bem
