// Preconditioners for the batched GMRES (block-Jacobi and learned).
#pragma once
#include <memory>

#include "common.cuh"
#include "gmres.cuh"

namespace bem {

// Leaves of the cluster tree and their near-field neighbours.
struct NearPattern {
    int64_t n = 0;
    int nc = 0;
    std::vector<int64_t> cl_off, cl_idx;  // leaf c holds cl_idx[cl_off[c] .. cl_off[c+1])
    std::vector<int32_t> nb_off, nb_d;    // neighbours d of leaf c (the first is c itself)
    std::vector<int64_t> nb_blk;          // storage offset of block (c, d), b_c x b_d column-major
    int64_t entries = 0;                  // block entries of one system
    std::vector<int32_t> pair_i, pair_j;  // every entry of the off-diagonal near blocks
    std::vector<int64_t> pair_dst;        // its storage index
    int64_t npairs = 0;
};

// The preconditioner network: FP32 master weights, their BF16-rounded copy
// used by the forward pass, Adam moments.
struct LearnedNet {
    DevBuf w, wbf, m1, m2;
    std::vector<float> w_host;
    int64_t step = 0;
    bool ready = false;
    void init(Context& c, uint64_t seed);
    void upload(Context& c);
    void refresh(Context& c);
};

int learned_num_params();
struct Forest;
// Leaves of the bodies' cluster trees (leaf size 64, built on the device) and
// their near neighbours (diag_only: each leaf with itself only, the
// block-Jacobi pattern); pats[b] belongs to bodies[b].
void build_patterns(Context& c, const std::vector<const Problem*>& bodies, std::vector<NearPattern>& pats,
                    bool diag_only);
// The pattern of one body of a forest built at leaf size 64, its leaves on
// parallel host threads when `parallel` is set (the same result either way;
// not from inside another host_parallel_for item).
void near_pattern(const Forest& F, int body, NearPattern& P, bool diag_only, bool parallel);
// Installs the preconditioner on the batch; returns the kind actually used
// (the learned form falls back to block-Jacobi when no network is available).
bem_precond precond_setup(Context& c, Problem& p, GmWorkspace& ws, bem_precond kind, const double* ks);
// Block steps per delayed trailing update of an LU factorization whose
// smallest system has nmin unknowns (4 or 8; the tuning table may choose 4
// where 8 is the default and 8 only from 4096 unknowns on).
int lu_group(const Context& c, int64_t nmin, int64_t nsys);
// Device bytes of the LU workspace per unknown of a system of n unknowns,
// beyond its FP32 factors (the most its group size may need).
double lu_bytes_per_unknown(int64_t n);
// Tensor-core LU of every operator of the batch, factored from its FP32
// rounding (lu32.cu).
void lu_precond_setup(Context& c, GmWorkspace& ws);
// Several bodies in a ragged batch: system s belongs to bodies[sys_body[s]].
bem_precond precond_setup_multi(Context& c, const std::vector<Problem*>& bodies, const std::vector<int>& sys_body,
                                GmWorkspace& ws, bem_precond kind, const double* ks);
double learned_train(Context& c, std::vector<Problem*>& probs, int steps, int nprobe, double lr, uint64_t seed,
                     std::vector<double>& losses);
void learned_mlp_eval(Context& c, int64_t P, const float* F, const float* dO, float* O, float* grad);
void learned_mlp_infer(Context& c, int64_t P, const float* F, float* O);
// Tensor-core inference (tc_mlp.cu): outputs to O (P x 2) and/or the learned
// entries s_p (o_1 + i o_2) to M[dst[p]].  With check = false the call
// neither clears nor reads the context's device error flag (the caller
// clears it before a series of calls and checks it after).
void mlp_infer_tc(Context& c, const LearnedNet& net, int64_t P, const float* F, float* O, const int64_t* dst,
                  const float* scale, float2* M, bool check = true);

}  // namespace bem
