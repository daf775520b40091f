// Batched restarted GMRES state (see gmres.cu).
#pragma once
#include "common.cuh"

namespace bem {

enum { MV_START = 0, MV_Q = 1, MV_CHECK = 2 };

struct GmState {
    double anorm, bnorm, tol, xnorm, error;
    int k, need_start, check, done, converged, m;  // m: this system's restart length (<= batch m)
    long long num_mv, iterations, restarts, max_restarts;
};

// Per-system layout of a ragged batch (systems of different sizes).
struct GmSys {
    int64_t n, lda, n_pad;
    size_t a_off;   // operator entries before this system's matrix
    size_t v_off;   // X, B, W
    size_t q_off;   // Q, Z
    size_t p_off;   // column-chunk partial sums
    size_t t_off;   // last-CTA tickets
    int64_t tile0;  // first CTA of this system in the flattened mat-vec grid
    int rb, cb;     // row blocks, column chunks
};

struct GmBatch {
    int nsys, m, ref_dotc, rb;
    int64_t n, n_pad, lda;  // uniform batch (sys == nullptr); ragged: largest n
    size_t mat_stride, qstride, small_stride;
    const GmSys* sys;   // ragged batch: per-system layout (nullptr: uniform)
    int64_t ntiles;     // ragged: CTAs of the flattened mat-vec grid
    int cb, pad;
    const void* A;      // nsys matrices (double2 or float2), column-major, leading dim lda
    double2* X;         // nsys x n solutions
    double2* B;         // nsys x n right-hand sides
    double2* Q;         // nsys x n x (m+1) Krylov bases
    double2* W;         // nsys x n operator outputs
    double2* part;      // column-chunk partial sums
    int* tickets;       // last-CTA counters
    double2* small;     // per-system Hessenberg / rotations
    GmState* st;
    double2* Z;         // flexible right preconditioning: Z[:, k] = M Q[:, k] (nullptr: none)
    // Gram-Schmidt of the mixed / refined forms across the whole GPU (null:
    // the single-CTA modified Gram-Schmidt of the reference form): per system,
    // partial dot products of every row chunk with the basis (gs_chunks x
    // (m + 1)) and partial squared norms (gs_chunks)
    double2* gs_part = nullptr;
    double* gs_norm = nullptr;
    int gs_chunks = 0;
    // split FP64 operators (refined form): every system's FP32 matrix (the
    // operator rounded to FP32, leading dimension lda) is followed, split_lo
    // float2 entries further on, by the FP32 rounding of the remainder, and
    // every mat-vec sums both in float-float (0: plain FP32 or FP64 operators)
    int64_t split_lo = 0;
};

// Whether the operator application of `mode` has work for a system.
__device__ __forceinline__ bool gm_apply_active(const GmBatch& bt, const GmState& s, int mode) {
    if (s.done) return false;
    if (mode == MV_START) return s.need_start != 0 && !(!bt.ref_dotc && s.restarts == 0);
    if (mode == MV_Q) return s.need_start == 0 && s.check == 0;
    return s.check != 0;  // MV_CHECK
}

// A system's sizes and offsets in either layout.
struct GmView {
    int64_t n, lda, n_pad;
    size_t a, v, q, p, t;
    int rb, cb;
};

__host__ __device__ __forceinline__ GmView gm_view(const GmBatch& bt, int s) {
    GmView v;
    if (bt.sys) {
        const GmSys& d = bt.sys[s];
        v.n = d.n; v.lda = d.lda; v.n_pad = d.n_pad;
        v.a = d.a_off; v.v = d.v_off; v.q = d.q_off; v.p = d.p_off; v.t = d.t_off;
        v.rb = d.rb; v.cb = d.cb;
    } else {
        v.n = bt.n; v.lda = bt.lda; v.n_pad = bt.n_pad;
        v.a = (size_t)s * bt.mat_stride; v.v = (size_t)s * bt.n; v.q = (size_t)s * bt.qstride;
        v.p = (size_t)s * bt.cb * bt.n_pad; v.t = (size_t)s * bt.rb;
        v.rb = bt.rb; v.cb = bt.cb;
    }
    return v;
}

struct GmSmall {
    double2 *hk1, *cs, *sn, *beta, *H, *y;
};

__host__ __device__ inline size_t gm_small_size(int m) {
    return (size_t)(m + 1) + m + m + (m + 1) + (size_t)(m + 1) * m + (m + 1);
}

__device__ inline GmSmall gm_small(const GmBatch& bt, int s) {
    double2* b = bt.small + (size_t)s * bt.small_stride;
    GmSmall g;
    int m = bt.m;
    g.hk1 = b;
    g.cs = g.hk1 + (m + 1);
    g.sn = g.cs + m;
    g.beta = g.sn + m;
    g.H = g.beta + (m + 1);
    g.y = g.H + (size_t)(m + 1) * m;
    return g;
}

struct GmWorkspace;
// Operator application hook (H-matrix): launches W_s = A_s v_s for `mode`,
// predicated on the state like the dense apply kernel.
typedef void (*GmApplyHook)(Context& ctx, GmWorkspace& ws, int mode, void* user);

struct GmWorkspace {
    GmBatch bt{};
    GmApplyHook hook = nullptr;
    void* hook_user = nullptr;
    // Preconditioner hook: launches Z_s[:, k] = M_s Q_s[:, k] for the systems
    // whose Krylov step is pending (same predicate as the MV_Q apply).
    GmApplyHook precond = nullptr;
    void* precond_user = nullptr;
    std::shared_ptr<void> precond_keep;  // owns the preconditioner data
    DevBuf zmem;
    DevBuf mem;
    // grow-only buffers of the context used instead of zmem / mem when set
    // (no allocation per solve)
    DevBuf* mem_pool = nullptr;
    DevBuf* z_pool = nullptr;
    DevBuf& memb() { return mem_pool ? *mem_pool : mem; }
    cudaEvent_t ev_p0 = nullptr, ev_p1 = nullptr;  // profiling: preconditioner application
    DevBuf& zb() { return z_pool ? *z_pool : zmem; }
    DevBuf init_args;
    std::vector<GmSys> sys_host;  // ragged layout (empty: uniform)
    bool fp32 = false;
    bool w_in_smem = false;
    int rb = 0, cb = 0;
    double* norm_part = nullptr;
    double* anorm = nullptr;
    // operator applied through `hook`: bytes streamed per system and mat-vec
    // and the profiling stage name of the Krylov mat-vec (0 / nullptr: the
    // dense operator's n^2 entries)
    double mv_bytes = 0;
    const char* mv_stage = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    int graph_chunk = 0, graph_rounds = 0;
    bool graph_loop = false;  // graph_exec is the whole solve (device-side loop)
    DevBuf rounds;            // rounds the solve graph ran
    int64_t launches_per_graph = 0;
    ~GmWorkspace();
};

void gm_prepare(Context& ctx, GmWorkspace& ws, int nsys, int64_t n, int m, const void* A, int64_t lda,
                size_t mat_stride, bool fp32, bool ref_dotc);
// Ragged batch: system s has size ns[s], leading dimension ldas[s] and its
// matrix at entry offset a_offs[s] of A.
void gm_prepare_ragged(Context& ctx, GmWorkspace& ws, const std::vector<int64_t>& ns,
                       const std::vector<int64_t>& ldas, const std::vector<size_t>& a_offs, int m, const void* A,
                       bool fp32);
size_t gm_prepare_external(Context& ctx, GmWorkspace& ws, int nsys, int64_t n, int m, const void* A, int64_t lda,
                           size_t mat_stride, bool fp32, bool ref_dotc, void* mem, size_t capacity);
// Entries of the Krylov basis Q (and of Z) over the whole batch.
size_t gm_q_total(const GmWorkspace& ws);
void gm_matrix_norms(Context& ctx, GmWorkspace& ws);
void gm_init(Context& ctx, GmWorkspace& ws, double tol, int64_t max_restarts);
// Per-system tolerance, restart count and restart length (m[s] <= batch m).
void gm_init_each(Context& ctx, GmWorkspace& ws, const std::vector<double>& tol,
                  const std::vector<int64_t>& max_restarts, const std::vector<int>& m);
void gm_launch_iteration(Context& ctx, GmWorkspace& ws, cudaEvent_t ev_q0, cudaEvent_t ev_q1);
void gm_read_states(Context& ctx, GmWorkspace& ws, std::vector<GmState>& out);
void gm_run(Context& ctx, GmWorkspace& ws, int chunk, int64_t max_total_iterations);

}  // namespace bem
