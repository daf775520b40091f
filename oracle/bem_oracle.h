/*
 * bem_oracle.h -- CPU FP64 restatement of the cc_abstemious BEM hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the oracle: the tests, the
 * smoke check and the CPU-baseline leg of the benchmark may call it; the
 * product path (cc_abstemious_gb300 + libbem_gb300.so) never links or calls it.
 *
 * Every function restates the reference algorithm and cites the reference
 * file:line it follows (paths relative to the cc_abstemious source tree).
 * Parity pins (checked by tests/test_oracle_golden.py):
 *   - src/tests/verification.rs:117-119 classical direct golden,
 *   - src/tests/verification.rs:146-147 classical GMRES golden,
 *   - src/tests/verification.rs:174-175 H-matrix + GMRES golden,
 *   - src/tests/verification.rs:202-204 Burton-Miller direct golden,
 *   - src/solve.rs:216-217 seeded 100x100 LU golden (needs the rand 0.9
 *     StdRng stream restated below),
 *   - the unit tests of aca.rs, h_matrix.rs, cluster.rs, block.rs, mesh_data.rs.
 *
 * Complex numbers are interleaved {re, im} doubles; matrices are column-major
 * with a leading dimension (nalgebra DMatrix layout).
 */
#ifndef BEM_ORACLE_H
#define BEM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- input (input_data.rs:9-92) ---------------------------------------- */
enum { OC_INTERIOR = 0, OC_EXTERIOR = 1 };
enum { OC_CLASSICAL = 0, OC_BURTON_MILLER = 1 };
enum { OC_DIRECT = 0, OC_ITERATIVE = 1, OC_HIERARCHICAL = 2 };
enum { OC_PLANE_WAVE = 0, OC_SPHERICAL_WAVE = 1 };
enum { OC_BC_PRESSURE = 0, OC_BC_NORMAL_VELOCITY = 1, OC_BC_IMPEDANCE = 2 };

/* Collocation point record (mesh_data.rs:71-77): x y z nx ny nz area wt. */
#define OC_CPT_STRIDE 8

typedef struct {
    double sound_speed, mass_density;
    int32_t problem_type, method_type, solver;
    int32_t incident_type, bc_type, output_total, output_pressure, pad0;
    double tolerance;
    int64_t max_iterations;
    double incident_vec[3];
    double incident_amp[2];
    double bc_value[2];
    /* H-matrix parameters: hard-coded leaf 32 / ACA tol 1e-4 in solve.rs:91-92,
       :119-120 and eta 4 in h_matrix.rs:136. */
    int64_t hm_leaf;
    double hm_eta;
    double hm_aca_tol;
    int64_t nfp;
    const double* field_points; /* nfp x 3 */
    int64_t n;
    const double* cpts;         /* n x OC_CPT_STRIDE */
    double frequency;
} oc_problem;

/* ---- mesh (mesh_data.rs:96-175) and collocation (elements.rs) ---------- */
typedef struct {
    int64_t nnodes;
    double* nodes;       /* 3 * nnodes */
    int64_t nelem;
    int64_t* body;       /* first integer of each CELLS row */
    int32_t* etype;      /* VTK cell type */
    int64_t* conn_off;   /* nelem + 1 */
    int64_t* conn;       /* node ids */
    int64_t nbodies;
    int32_t status;      /* 0 ok, else parse error code */
} oc_mesh;

int oc_read_vtk(const char* path, oc_mesh* out);
void oc_mesh_free(oc_mesh* m);
/* Returns number of collocation points of body `body_index` (1-based);
   writes them when cpts != NULL.  Negative on error. */
int64_t oc_collocation(const oc_mesh* m, int64_t body_index, double* cpts);

/* ---- frequency list (tools.rs:1-24) ------------------------------------ */
int oc_linspace(double start, double end, int64_t n, double* out);
int oc_logspace(double start, double end, int64_t n, double* out);

/* ---- kernels and matrices (influence_matrix.rs) ------------------------ */
void oc_greens(double k, const double* x, const double* nx, const double* y,
               const double* ny, int bm, double* g, double* h);
void oc_gh(const oc_problem* p, int64_t i, int64_t j, double* g, double* h);
void oc_dense_surface(const oc_problem* p, double* H, double* G, int64_t ld, int nthreads);
void oc_dense_field(const oc_problem* p, double* M, double* L, int64_t ld);
void oc_lhs_factors(const oc_problem* p, double* alpha, double* beta);
void oc_rhs_factors(const oc_problem* p, double* gamma, double* delta);
/* side: 0 = RHS, 1 = LHS.  Exactly one of ni, nj must be 1. */
int oc_row_or_column(const oc_problem* p, const int64_t* Ir, int64_t ni,
                     const int64_t* Jc, int64_t nj, int side, double* out);

/* ---- incident wave (incident_wave.rs) ---------------------------------- */
void oc_incident_surface(const oc_problem* p, double* rhs_inc);
void oc_incident_field(const oc_problem* p, double* phi_inc_fp);

/* ---- solvers (solve.rs, gmres.rs) -------------------------------------- */
int oc_lu_solve(int64_t n, const double* A, int64_t lda, double* b);
typedef struct {
    int64_t num_mv;
    int64_t restarts;
    double error;
    int32_t flag;   /* 0 error, 1 tolerance, 2 iterations */
    int32_t pad;
} oc_gmres_report;
int oc_gmres_dense(int64_t n, const double* A, int64_t lda, int64_t max_it,
                   double tol, double* x, oc_gmres_report* rep);
/* (phi, vn) on the surface; solver chosen by p->solver (solve.rs:11-22). */
int oc_solve_for_surface(const oc_problem* p, const double* rhs_inc,
                         double* phi, double* vn, oc_gmres_report* rep, int nthreads);
void oc_get_field(const oc_problem* p, const double* M, const double* L, int64_t ld,
                  const double* phi, const double* vn, const double* phi_inc_fp,
                  double* out);
void oc_convert_to_pressure(const oc_problem* p, double* v, int64_t n);
/* One iteration of the frequency loop of analysis.rs:87-111 (without the
   pressure conversion of postprocess.rs:70-79, applied by the caller). */
int oc_run_frequency(const oc_problem* p, double* phi, double* vn,
                     double* fp_scattered, double* fp_incident,
                     oc_gmres_report* rep, int nthreads);

/* ---- H-matrix (h_matrix.rs, cluster.rs, block.rs, aca.rs) -------------- */
typedef struct oc_hmatrix oc_hmatrix;
/* Generic generator: fills out with row i over columns J (nj) when ni == 1,
   or column j over rows I when nj == 1. */
typedef void (*oc_rowcol_fn)(void* ctx, const int64_t* Ir, int64_t ni,
                             const int64_t* Jc, int64_t nj, double* out);
oc_hmatrix* oc_hmatrix_build(int64_t n, const double* points, int64_t point_stride,
                             int64_t leaf, double eta, double tol,
                             oc_rowcol_fn gen, void* ctx);
void oc_hmatrix_free(oc_hmatrix* h);
double oc_hmatrix_norm(const oc_hmatrix* h);
void oc_hmatrix_gemv(const oc_hmatrix* h, const double* alpha, const double* x,
                     const double* beta, double* b);
void oc_hmatrix_to_full(const oc_hmatrix* h, double* A, int64_t lda);
/* stats: [0] admissible count, [1] inadmissible count, [2] stored entries,
   [3] sum of ranks */
void oc_hmatrix_stats(const oc_hmatrix* h, int64_t* stats);
/* Leaf-block export (device upload / tests): for block b returns
   rows, cols, admissible flag and rank. */
int64_t oc_hmatrix_num_blocks(const oc_hmatrix* h);
int oc_gmres_hmatrix(const oc_hmatrix* h, int64_t max_it, double tol, double* x,
                     oc_gmres_report* rep);

/* cluster / block tree (cluster.rs:35-105, block.rs:38-96) */
typedef struct {
    int64_t nblocks;
    int64_t* row_off;   /* nblocks + 1 */
    int64_t* rows;
    int64_t* col_off;
    int64_t* cols;
    int32_t* admissible;
    double root_diameter;
} oc_blocklist;
int oc_block_list(int64_t n, const double* points, int64_t point_stride,
                  int64_t leaf, double eta, oc_blocklist* out);
void oc_blocklist_free(oc_blocklist* b);
/* Path lookup used by block.rs:104-115: admissible flag of the block reached by
   following child indices path[0..depth) from the root; -1 if absent. */
int oc_block_tree_path_admissible(int64_t n, const double* points, int64_t point_stride,
                                  int64_t leaf, double eta, const int32_t* path, int depth);

/* ACA on a generic generator (aca.rs:23-136); returns rank, fills U (m x r)
   and V (n x r) when non-NULL (capacity min(m,n) columns), norm estimate. */
int64_t oc_aca(int64_t m, int64_t n, double tol, oc_rowcol_fn gen_row_col, void* ctx,
               double* U, double* V, double* norm_est);

/* ---- rand 0.9 StdRng restatement (ChaCha12, rand_core seed_from_u64) --- */
typedef struct {
    uint32_t key[8];
    uint64_t counter;
    uint32_t buf[64];
    int32_t idx;
} oc_stdrng;
void oc_stdrng_seed(oc_stdrng* r, uint64_t seed);
uint32_t oc_stdrng_u32(oc_stdrng* r);
uint64_t oc_stdrng_u64(oc_stdrng* r);
double oc_stdrng_f64(oc_stdrng* r);
/* rand 0.9 Uniform::new_inclusive(lo, hi) over usize, .sample() */
uint64_t oc_uniform_usize_incl(oc_stdrng* r, uint64_t lo, uint64_t hi);
/* solve.rs:194-209 generate_random_ab (column-major m x n, and b of length n) */
void oc_generate_random_ab(int64_t m, int64_t n, uint64_t seed, double* A, double* b);

#ifdef __cplusplus
}
#endif
#endif
