// Mixed form over H-matrix operators (hmixed.cu).
#pragma once
#include <memory>

#include "common.cuh"
#include "gmres.cuh"

namespace bem {

struct HMixed;
struct HMixedStats {
    int64_t blocks = 0, admissible = 0, clusters = 0;
    int64_t store_entries = 0, dense_entries = 0, lowrank_entries = 0;  // complex FP32 entries, all operators
};

// The operators of frequencies F0 .. F0 + nops of p (lhs factors), each
// ACA-compressed in FP64 and repacked as FP32 in cluster order; R systems
// (incident waves) share each operator: system s uses operator s / R.
std::shared_ptr<HMixed> hmixed_build(Context& c, Problem& p, int64_t F0, int64_t nops, int R);
// Makes H the batch's operator (GMRES apply hook and stopping-test norms).
void hmixed_attach(Context& c, GmWorkspace& ws, const std::shared_ptr<HMixed>& H);
// Block-Jacobi preconditioner from the dense diagonal leaves; false when a
// leaf is larger than 64 (no preconditioner installed).
bool hmixed_block_jacobi(Context& c, GmWorkspace& ws, const std::shared_ptr<HMixed>& H);
HMixedStats hmixed_stats(const HMixed& H);

}  // namespace bem
