/*
 * bem.h -- C ABI of libbem_gb300.so, the GB300 (sm_103a) implementation of the
 * cc_abstemious BEM hot path.
 *
 * The reference is a pure-Rust crate whose hot-path boundary is its module API
 * (influence_matrix / solve / postprocess, driven by analysis.rs).  Every entry
 * point below replaces one of those functions; the comment gives the reference
 * file:line.  A Rust crate binds these with `extern "C"` declarations of the
 * same signatures.
 *
 * Conventions
 *  - Complex values are interleaved {re, im} doubles (bem_cplx), matching
 *    num_complex::Complex<f64>.  Matrices are column-major with a leading
 *    dimension, matching nalgebra DMatrix<Complex<f64>>.
 *  - The caller owns every buffer.  `mem` says whether matrix/vector pointers
 *    are host (BEM_MEM_HOST) or CUDA device (BEM_MEM_DEVICE) memory of the
 *    context's device.
 *  - Calls are synchronous: results are ready when the call returns.  One
 *    context per host thread.
 *  - Errors never abort: every call returns a bem_status and the context keeps
 *    a message for bem_last_error().  The reference panics (unwrap) or logs
 *    and continues instead.
 */
#ifndef BEM_GB300_H
#define BEM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BEM_API __attribute__((visibility("default")))

typedef struct { double re, im; } bem_cplx;

typedef enum {
    BEM_OK = 0,
    BEM_ERR_BAD_INPUT = 1,     /* malformed JSON/VTK, bad sizes or indices */
    BEM_ERR_SINGULAR = 2,      /* zero pivot in an LU factorisation */
    BEM_ERR_NOT_CONVERGED = 3, /* iterative solver ran out of iterations */
    BEM_ERR_NAN = 4,           /* NaN produced (e.g. zero spherical-wave origin) */
    BEM_ERR_OOM = 5,           /* device allocation failed */
    BEM_ERR_CUDA = 6,          /* CUDA runtime error */
    BEM_ERR_TIMEOUT = 7        /* a bounded device-side wait gave up */
} bem_status;

typedef enum { BEM_MEM_HOST = 0, BEM_MEM_DEVICE = 1 } bem_mem;

/* influence_matrix.rs:164-167 EqnSide */
typedef enum { BEM_SIDE_RHS = 0, BEM_SIDE_LHS = 1 } bem_side;

/* Execution form of bem_run / bem_solve_for_surface.
 *  PLAIN_FP64: drop-in form; every stage in FP64 following the reference
 *              algorithms (LU, restarted GMRES, ACA H-matrix).
 *  MIXED:      all frequencies batched; FP32 assembly with accurate phase
 *              reduction, FP64 restarted GMRES over the FP32 operator with
 *              compensated mat-vecs, optional preconditioner; each result
 *              reports its error against an FP64 LU when requested.
 *  REFINED:    as MIXED, but every operator is carried at FP64 accuracy
 *              (assembled in float-float and stored as its FP32 rounding plus
 *              the FP32 remainder, applied in float-float: residuals and the
 *              answer at FP64 accuracy, for operators whose condition number
 *              makes FP32 storage miss 1e-6), while the preconditioner is
 *              built from its FP32 rounding (the tensor-core LU of
 *              BEM_PRECOND_LU).
 *  MIXED_ROUNDED: as MIXED, over operators rounded to FP32 once from their
 *              float-float values (the REFINED assembly without the
 *              remainder): about half the FP32 operator error of MIXED at
 *              several times its assembly cost, for operators whose
 *              conditioning puts MIXED just above the required accuracy.
 *              Inputs with row sums on the right-hand side (nonzero
 *              pressure or velocity conditions) use the MIXED assembly. */
typedef enum { BEM_FORM_PLAIN_FP64 = 0, BEM_FORM_MIXED = 1, BEM_FORM_REFINED = 2, BEM_FORM_MIXED_ROUNDED = 3 } bem_form;

/* Preconditioners of the mixed form (no counterpart in the reference, whose
 * GMRES is unpreconditioned, gmres.rs:80-140).  Flexible right
 * preconditioning; the FP64 residual decides convergence, so a preconditioner
 * changes the iteration count, never the answer.
 *  BLOCK_JACOBI: inverses of the diagonal cluster-leaf blocks.
 *  LEARNED:      block-Jacobi plus a network-predicted near-field correction
 *                (falls back to BLOCK_JACOBI without a trained network).
 *  LU:           a tensor-core LU (no pivoting) of each operator's FP32
 *                rounding (TF32 panels, FP16 trailing updates with FP32
 *                accumulation), applied by blocked triangular solves; for
 *                hard systems (high frequency, fine meshes) where GMRES
 *                alone stalls. */
typedef enum {
    BEM_PRECOND_NONE = 0,
    BEM_PRECOND_BLOCK_JACOBI = 1,
    BEM_PRECOND_LEARNED = 2,
    BEM_PRECOND_LU = 3
} bem_precond;

typedef struct {
    int64_t num_mv;         /* matrix-vector products (gmres.rs:66) */
    int64_t restarts;       /* restart cycles started */
    int64_t iterations;     /* Arnoldi steps */
    double backward_error;  /* final ||r|| / (||A|| ||x|| + ||b||) */
    double rel_err_vs_lu;   /* ||x - x_LU64|| / ||x_LU64||, -1 if not computed */
    double seconds;         /* wall time of the call */
    int32_t flag;           /* 0 error, 1 tolerance reached, 2 iterations exhausted, 3 direct */
    int32_t precond;        /* bem_precond used */
} bem_solve_report;

typedef struct bem_ctx bem_ctx;
typedef struct bem_problem bem_problem;
typedef struct bem_hmatrix bem_hmatrix;

/* Parsed UserInput (input_data.rs:80-92), for inspection. */
typedef struct {
    double sound_speed, mass_density;
    int32_t problem_type;    /* 0 Interior, 1 Exterior */
    int32_t method_type;     /* 0 Classical, 1 BurtonMiller */
    int32_t solver;          /* 0 Direct, 1 Iterative, 2 Hierarchical */
    int32_t incident_type;   /* 0 PlaneWave, 1 SphericalWave */
    int32_t bc_type;         /* 0 Pressure, 1 NormalVelocity, 2 Impedance */
    int32_t output_total;    /* OutputType::Total */
    int32_t output_pressure; /* OutputField::Pressure */
    int32_t body_index;
    double tolerance;
    int64_t max_iterations;
    double incident_vec[3];
    double incident_amp[2];
    double bc_value[2];
    int64_t hm_leaf;         /* additive extension keys, defaults 32 / 4.0 / 1e-4 */
    double hm_eta;
    double hm_aca_tol;
    int64_t num_eqn;
    int64_t num_field_points;
    int64_t num_frequencies;
    int64_t mesh_elements;
    int64_t mesh_nodes;
    int64_t mesh_bodies;
    int64_t num_rhs;         /* incident_wave + the extension key additional_incident_waves */
} bem_problem_info;

/* ---- context ---------------------------------------------------------- */
BEM_API bem_status bem_ctx_create(int device, bem_ctx** out);
BEM_API void bem_ctx_destroy(bem_ctx* ctx);
BEM_API const char* bem_last_error(const bem_ctx* ctx);
/* Number of kernels this context has launched (instrumentation). */
BEM_API int64_t bem_ctx_kernel_launches(const bem_ctx* ctx);
BEM_API const char* bem_version(void);
/* Per-stage CUDA-event timing of bem_run (instrumentation; no reference
 * counterpart).  Profiling runs the GMRES iteration by iteration so that every
 * Krylov mat-vec launch is bracketed by events on the context's stream. */
BEM_API bem_status bem_ctx_set_profiling(bem_ctx* ctx, int on);
/* The context's CUDA stream (cudaStream_t), so callers can order their own
 * work or record CUDA events around library calls. */
BEM_API void* bem_ctx_stream(const bem_ctx* ctx);
BEM_API int64_t bem_ctx_profile_count(const bem_ctx* ctx);
BEM_API bem_status bem_ctx_profile_get(const bem_ctx* ctx, int64_t i, char* name, int64_t name_len,
                                       double* ms, int64_t* launches, double* bytes);

/* ---- launch tuning (no reference counterpart) ------------------------- */
/* Launch parameters of the hot kernels (the trailing update's tile raster,
 * the Krylov mat-vec's load batch, the FP32 assembly's occupancy) come from a
 * tuning table keyed by problem size and number of systems, written by the
 * offline sweep cc_abstemious_gb300/tune.py.  A context reads tuning.json
 * beside the library at creation when it exists (the environment variable
 * BEM_TUNING_FILE names another file, or "none" for the built-in defaults).
 * bem_ctx_load_tuning reads a table (NULL: back to the defaults);
 * bem_ctx_set_tuning forces one parameter (value < 0 removes the override);
 * bem_ctx_get_tuning returns the value a launch of that size would use. */
BEM_API bem_status bem_ctx_load_tuning(bem_ctx* ctx, const char* path);
BEM_API bem_status bem_ctx_set_tuning(bem_ctx* ctx, const char* kernel, const char* param, int value);
BEM_API int bem_ctx_get_tuning(const bem_ctx* ctx, const char* kernel, const char* param, int64_t n, int64_t nsys);
/* The file the context's table was read from ("" for the built-in defaults). */
BEM_API const char* bem_ctx_tuning_source(const bem_ctx* ctx);

/* ---- input and preprocessing ------------------------------------------ */
/* analysis.rs:50-53 input_from_string + preprocess.rs:104-124 preprocess.
 * base_dir (may be NULL) resolves a relative mesh_file; the reference resolves
 * it against the working directory. */
BEM_API bem_status bem_problem_from_json(bem_ctx* ctx, const char* json, const char* base_dir,
                                         bem_problem** out);
/* analysis.rs:42-48 input_from_file (input_data.rs:94-103). */
BEM_API bem_status bem_problem_from_file(bem_ctx* ctx, const char* path, bem_problem** out);
BEM_API void bem_problem_destroy(bem_problem* p);
BEM_API bem_status bem_problem_get_info(const bem_problem* p, bem_problem_info* out);
/* preprocess.rs:155-167 frequency list (tools.rs:1-24). */
BEM_API bem_status bem_problem_frequencies(const bem_problem* p, double* out);
/* preprocess.rs:34 PreData::set_frequency_index */
BEM_API bem_status bem_problem_set_frequency_index(bem_problem* p, int64_t index);
/* Collocation points x y z nx ny nz area wt (n x 8, row-major), computed on the
 * device by the collocation kernel: elements.rs:172-180 via
 * preprocess.rs:126-153. */
BEM_API bem_status bem_collocation(bem_ctx* ctx, const bem_problem* p, double* out);

/* The operators A_f = alpha_f H_f + beta_f G_f of frequencies f0 .. f0 + nf - 1
 * (the factors of influence_matrix.rs:130-162) as the batched forms assemble
 * them, for checking them against bem_get_dense_surface_matrices: kind 0 the
 * mixed form's single-precision assembly, kind 1 the refined form's split
 * float-float assembly (FP32 rounding + FP32 remainder, summed here in FP64),
 * kind 2 the MIXED_ROUNDED form's operator (that FP32 rounding alone).
 * A (host) receives nf matrices of n x n, column-major, leading dimension lda,
 * lda * n entries apart.  No reference counterpart (the reference assembles
 * FP64 only, influence_matrix.rs:64-98). */
BEM_API bem_status bem_assemble_operator(bem_ctx* ctx, const bem_problem* p, int kind, int64_t f0, int64_t nf,
                                         bem_cplx* A, int64_t lda);

/* ---- influence matrices (influence_matrix.rs) ------------------------- */
/* influence_matrix.rs:64-98 get_dense_surface_matrices -> (H, G), n x n. */
BEM_API bem_status bem_get_dense_surface_matrices(bem_ctx* ctx, const bem_problem* p,
                                                  bem_cplx* H, bem_cplx* G, int64_t ld, bem_mem mem);
/* influence_matrix.rs:101-127 get_dense_field_matrices -> (M, L), nfp x n. */
BEM_API bem_status bem_get_dense_field_matrices(bem_ctx* ctx, const bem_problem* p,
                                                bem_cplx* M, bem_cplx* L, int64_t ld, bem_mem mem);
/* influence_matrix.rs:170-193 get_surface_row_or_column: exactly one of ni, nj
 * must be 1; out has max(ni, nj) entries.  Index arrays are host memory. */
BEM_API bem_status bem_get_surface_row_or_column(bem_ctx* ctx, const bem_problem* p,
                                                 const int64_t* I, int64_t ni,
                                                 const int64_t* J, int64_t nj,
                                                 bem_side side, bem_cplx* out);

/* The mixed form's single-precision system matrix alpha H + beta G
 * (influence_matrix.rs:130-146 factors) at the current frequency, as
 * interleaved {re, im} floats, n x n column-major, host memory. */
BEM_API bem_status bem_get_system_matrix_fp32(bem_ctx* ctx, const bem_problem* p, float* A, int64_t ld);

/* ---- incident wave (incident_wave.rs) --------------------------------- */
/* incident_wave.rs:7-63 get_incident_surface (n entries, host memory). */
BEM_API bem_status bem_get_incident_surface(bem_ctx* ctx, const bem_problem* p, bem_cplx* rhs_inc);
/* incident_wave.rs:66-99 get_incident_field (nfp entries, host memory). */
BEM_API bem_status bem_get_incident_field(bem_ctx* ctx, const bem_problem* p, bem_cplx* phi_inc_fp);

/* ---- solvers (solve.rs, gmres.rs) ------------------------------------- */
/* solve.rs:11-22 solve_for_surface (dense direct / iterative / hierarchical
 * per the problem's solver), plain FP64 form.  Host vectors of length n. */
BEM_API bem_status bem_solve_for_surface(bem_ctx* ctx, const bem_problem* p, const bem_cplx* rhs_inc,
                                         bem_cplx* phi, bem_cplx* vn, bem_solve_report* report);
/* solve.rs:166-171 solve_lu: x (length n) is overwritten by A^-1 x. */
BEM_API bem_status bem_solve_lu(bem_ctx* ctx, int64_t n, const bem_cplx* A, int64_t lda,
                                bem_cplx* x, bem_mem mem);
/* gmres.rs:35-59 GMRES::solve on a dense matrix (zero initial guess). */
BEM_API bem_status bem_gmres_solve(bem_ctx* ctx, int64_t n, const bem_cplx* A, int64_t lda,
                                   int64_t max_it, double tol, bem_cplx* x,
                                   bem_solve_report* report, bem_mem mem);
/* No counterpart in the reference.  The dense GMRES of bem_gmres_solve, with A
 * and x (in: b, out: solution) in device memory, that allocates no device
 * memory: its working memory is a fixed 8 MiB array in the library's device
 * image, held by every GPU that loads the library until the process exits.  For
 * callers that cannot allocate device memory at solve time, such as
 * applications that give all device memory to their own pool up front or run a
 * fixed-budget loop, where a cudaMalloc would synchronise the device or fail.
 * Limit: n up to 4096 at any iteration limit; sizes whose workspace exceeds the
 * array are rejected with BEM_ERR_BAD_INPUT before any work is issued.  The
 * first call on each device looks up the array's device address and keeps it
 * for the life of the process; make that first call before any stream capture,
 * and do not use this entry point after a cudaDeviceReset in the same process.
 * The call synchronises the context's stream after every iteration (it reads
 * the convergence state on the host) and fills report->seconds like
 * bem_gmres_solve.  Every call uses the same array, so calls that overlap on
 * the GPU (other threads, other streams) race. */
BEM_API bem_status bem_gmres_solve_noalloc(bem_ctx* ctx, int64_t n, const bem_cplx* A, int64_t lda,
                                           int64_t max_it, double tol, bem_cplx* x, bem_solve_report* report);
/* solve.rs:173-185 get_field: out = [phi_inc if Total] - M phi + L vn. */
BEM_API bem_status bem_get_field(bem_ctx* ctx, const bem_problem* p, const bem_cplx* M,
                                 const bem_cplx* L, int64_t ld, const bem_cplx* phi,
                                 const bem_cplx* vn, const bem_cplx* phi_inc_fp,
                                 bem_cplx* out, bem_mem mem);
/* Fused field evaluation: influence_matrix.rs:101-127 + solve.rs:173-185
 * evaluated without storing M and L.  Host vectors. */
BEM_API bem_status bem_evaluate_field(bem_ctx* ctx, const bem_problem* p, const bem_cplx* phi,
                                      const bem_cplx* vn, const bem_cplx* phi_inc_fp, bem_cplx* out);
/* postprocess.rs:83-87 convert_phi_to_pressure_vec: v *= i omega rho. */
BEM_API bem_status bem_convert_to_pressure(const bem_problem* p, double frequency, bem_cplx* v, int64_t n);

/* ---- output (postprocess.rs:15-67) --------------------------------------- */
/* postprocess.rs:15-44 write_results_at_frequency: one CSV record per field
 * point (index, x, y, z, pre_re/vpo_re, pre_im/vpo_im, inc_re, inc_im) of one
 * frequency's results (nfp entries each, host memory, as bem_run leaves them:
 * pressure or potential).  path NULL: the input's output.file.  Numbers as
 * Rust's f64 Display writes them (see bem_format_f64); records end in "\n".
 * ctx (may be NULL) receives the error message. */
BEM_API bem_status bem_write_results_at_frequency(bem_ctx* ctx, const bem_problem* p, const char* path,
                                                  const bem_cplx* scattered, const bem_cplx* incident);
/* postprocess.rs:46-67 write_results_at_point: one CSV record per frequency
 * (freq, pre_re/vpo_re, pre_im/vpo_im, inc_re, inc_im) for field point
 * `index`; scattered and incident are num_frequencies x nfp (field point
 * fastest, one wave), as bem_run fills them. */
BEM_API bem_status bem_write_results_at_point(bem_ctx* ctx, const bem_problem* p, const char* path, int64_t index,
                                              const bem_cplx* scattered, const bem_cplx* incident);
/* The number format of the CSV writers: Rust's `f64::to_string()` (shortest
 * round-trip digits, positional notation, no ".0" on integral values, "NaN",
 * "inf").  Writes at most len - 1 characters and a terminating NUL into buf;
 * returns the full length (or -1). */
BEM_API int64_t bem_format_f64(double v, char* buf, int64_t len);

/* ---- driver (analysis.rs:57-118) --------------------------------------- */
/* Runs every frequency of the problem.  scattered and incident are
 * (num_rhs x num_frequencies x nfp) row-major host arrays (field point
 * fastest; num_rhs = 1 unless the input lists additional_incident_waves, in
 * which case every wave is solved with the same operators: the mixed and
 * refined forms assemble and factor each frequency once) and
 * receive the pressure (or velocity potential) as postprocess.rs:70-79
 * leaves them.  reports: num_frequencies entries or NULL.  With
 * check_vs_lu != 0 each report carries its error against an FP64 LU solve of
 * the same operator (costly; outside any timed region). */
/* reports: num_rhs x num_frequencies entries (wave-major) or NULL. */
BEM_API bem_status bem_run(bem_ctx* ctx, bem_problem* p, bem_form form, bem_precond precond,
                           bem_cplx* scattered, bem_cplx* incident, bem_solve_report* reports,
                           int check_vs_lu);
/* Several bodies in one batch (mixed form).  No counterpart in the reference,
 * which runs one Analysis per body (analysis.rs:87-111): here every frequency
 * of every body is assembled by one multi-body launch and all systems are
 * solved by one batched GMRES over systems of different sizes.  scattered[b],
 * incident[b] and reports[b] are the per-body arrays of bem_run (the pointer
 * arrays, or any entry, may be NULL).  max_operator_bytes bounds the operators
 * held at once (bodies are grouped into chunks; 0: a share of the free device
 * memory).  Bodies with a classical formulation and a pressure condition keep
 * an FP64 operator and run one by one as in bem_run.  Only the first incident
 * wave of each body is solved (additional_incident_waves: bem_run). */
BEM_API bem_status bem_run_batch(bem_ctx* ctx, bem_problem* const* problems, int nprob, bem_precond precond,
                                 bem_cplx* const* scattered, bem_cplx* const* incident,
                                 bem_solve_report* const* reports, int check_vs_lu,
                                 int64_t max_operator_bytes);
/* Surface solutions of the last bem_run (n per system; wave-major, then
 * frequency: num_rhs x num_frequencies x n). */
BEM_API bem_status bem_last_surface(bem_ctx* ctx, const bem_problem* p, bem_cplx* phi, bem_cplx* vn);

/* ---- learned preconditioner (no counterpart in the reference) ------------ */
/* Near-field block preconditioner M = blockdiag(A_cc)^-1 + C where the entries
 * of C on the near off-diagonal leaf blocks come from a 3-layer MLP (width 128,
 * BF16 weights/activations, FP32 accumulation) over pair geometry and ka.
 * bem_learned_train trains the context's network on the GPU on the operators of
 * the given problems (all their frequencies) by minimising, per system,
 * E ||A M z - z||^2 / ||z||^2 over random probes relative to the same loss
 * with block-Jacobi alone (so systems of every wavenumber weigh alike); losses
 * (steps entries, may be NULL) receive that relative loss per step (1: no
 * better than block-Jacobi).  Used by bem_run with BEM_PRECOND_LEARNED. */
BEM_API bem_status bem_learned_train(bem_ctx* ctx, bem_problem* const* problems, int nproblems, int steps,
                                     int nprobe, double lr, uint64_t seed, double* losses);
BEM_API int64_t bem_learned_num_params(void);
BEM_API bem_status bem_learned_get_weights(bem_ctx* ctx, float* w);
BEM_API bem_status bem_learned_set_weights(bem_ctx* ctx, const float* w);
/* Network forward on P feature rows (P x 16) -> outputs (P x 2); with dO
 * (P x 2) also the parameter gradients of sum(dO * O) (num_params floats). */
BEM_API bem_status bem_learned_mlp_eval(bem_ctx* ctx, int64_t P, const float* features, const float* dO,
                                        float* out, float* grad);
/* Network outputs (P x 2) by the tensor-core (tcgen05) inference kernel that
 * bem_run uses to emit the learned preconditioner entries. */
BEM_API bem_status bem_learned_mlp_infer(bem_ctx* ctx, int64_t P, const float* features, float* out);

/* ---- LU preconditioner kernels (instrumentation; no reference counterpart) */
/* The LU preconditioner's factorization (tensor-core panel and trailing updates,
 * no pivoting, blocks of 128) and one application z = U^-1 L^-1 q, on
 * caller-given operators, with everything read back, so the device kernels
 * can be compared entry by entry with an FP64 LU.  System s has n[s] unknowns
 * and its complex FP32 matrix (interleaved {re, im}, column-major, leading
 * dimension ld[s]) at complex offset a_off[s] of the host array A (a_entries
 * complex entries); ld[s] and a_off[s] are multiples of 64; systems with the
 * same a_off share one operator (several right-hand sides).  F (may be NULL)
 * receives A's layout holding, per block row/column of 128, L21 below the
 * diagonal blocks, U12 above them and the updated diagonal blocks
 * (L_bb U_bb).  D (may be NULL; d_entries complex entries) receives per
 * factored operator, in order of first appearance, one 128 x 128 column-major
 * tile per diagonal block: L_bb^-1 strictly below the diagonal (unit diagonal
 * implied) and U_bb^-1 on and above it.  q and z (may be NULL) are the
 * systems' vectors back to back (sum of n[s] complex doubles); z receives
 * M q.  small_pivots (may be NULL) receives the number of pivots replaced. */
BEM_API bem_status bem_lu32_factor_apply(bem_ctx* ctx, int nsys, const int64_t* n, const int64_t* ld,
                                         const int64_t* a_off, int64_t a_entries, const float* A, float* F,
                                         float* D, int64_t d_entries, const bem_cplx* q, bem_cplx* z,
                                         int* small_pivots);

/* ---- Cluster and block trees (cluster.rs:35-105, block.rs:38-93) ------- */
/* Cluster::new_from (cluster.rs:23-31) and BlockList::new_from over
 * BlockTree::new_from (block.rs:20-28, :76-93) for nsets point sets at once,
 * built on the device.  Set s has npts[s] points, `stride` doubles per point
 * (x y z first), the sets back to back in pts (host memory).
 *   perm (sum of npts entries): each set's point indices (0-based within the
 *     set) in cluster order, the sets back to back;
 *   leaves (3 per leaf: set, begin, end): the leaf clusters depth-first, each
 *     the range begin .. end - 1 of its set's part of perm;
 *   blocks (6 per block: set, row begin, row end, column begin, column end,
 *     admissible): the block-tree leaves in the reference's flattening order
 *     (eta < 0: no block tree, *nblocks = 0);
 *   root_diam (nsets entries, may be NULL): each root's box diagonal.
 * *nleaves and *nblocks receive the counts; when one exceeds its capacity the
 * call returns BEM_ERR_BAD_INPUT without writing leaves and blocks, and the
 * caller may retry with the counts.  Coincident points that cannot be
 * separated are BEM_ERR_BAD_INPUT (the reference recurses without end). */
BEM_API bem_status bem_cluster_tree(bem_ctx* ctx, int nsets, const int64_t* npts, const double* pts, int64_t stride,
                                    int64_t leaf, double eta, int64_t* perm, int64_t* leaves, int64_t leaf_cap,
                                    int64_t* nleaves, int64_t* blocks, int64_t block_cap, int64_t* nblocks,
                                    double* root_diam);

/* ---- H-matrix (h_matrix.rs, aca.rs, cluster.rs, block.rs) -------------- */
/* h_matrix.rs:127-148 HMatrix::new_from over the problem's collocation points
 * for the given side (leaf, eta and ACA tolerance from the problem). */
BEM_API bem_status bem_hmatrix_build(bem_ctx* ctx, const bem_problem* p, bem_side side, bem_hmatrix** out);
BEM_API void bem_hmatrix_destroy(bem_hmatrix* h);
/* h_matrix.rs:218-234 gemv: b = alpha H x + beta b (host vectors). */
BEM_API bem_status bem_hmatrix_gemv(bem_ctx* ctx, const bem_hmatrix* h, bem_cplx alpha, const bem_cplx* x,
                                    bem_cplx beta, bem_cplx* b);
/* h_matrix.rs:150 get_norm (sum of leaf Frobenius norms / ACA estimates). */
BEM_API double bem_hmatrix_norm(const bem_hmatrix* h);
/* [0] admissible leaves, [1] inadmissible leaves, [2] stored entries, [3] sum of ranks */
BEM_API bem_status bem_hmatrix_stats(const bem_hmatrix* h, int64_t* stats4);
/* h_matrix.rs:236-246 to_full (n x n column-major, host). */
BEM_API bem_status bem_hmatrix_to_full(bem_ctx* ctx, const bem_hmatrix* h, bem_cplx* A, int64_t lda);

#ifdef __cplusplus
}
#endif
#endif
