// Internal definitions shared by the translation units of libbem_gb300.so.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <functional>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/bem.h"

namespace bem {

// ---------------------------------------------------------------------------
// Errors: C-ABI functions catch bem::Error and return its status.
struct Error : std::runtime_error {
    bem_status status;
    Error(bem_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

#define BEM_CUDA(call)                                                                      \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess)                                                              \
            throw ::bem::Error(e_ == cudaErrorMemoryAllocation ? BEM_ERR_OOM : BEM_ERR_CUDA, \
                               std::string(#call) + ": " + cudaGetErrorString(e_));         \
    } while (0)

#define BEM_CHECK_LAUNCH(ctx) \
    do { (ctx)->launches++; BEM_CUDA(cudaGetLastError()); } while (0)

inline void require(bool ok, const std::string& msg, bem_status s = BEM_ERR_BAD_INPUT) {
    if (!ok) throw Error(s, msg);
}

// f(i) for every i in [0, n) on the process's host worker threads, the
// calling thread among them, items handed out one at a time; returns when all
// are done and rethrows the first exception an item raised.  Calls for
// distinct i must be safe to run at the same time.  Calls from several host
// threads take the workers in turn; an item must not call it again (it would
// wait for itself).
void host_parallel_for(int64_t n, const std::function<void(int64_t)>& f);

// ---------------------------------------------------------------------------
// Input model: UserInput of input_data.rs:80-92.
struct UserInput {
    std::string mesh_file;
    int64_t body_index = 0;
    int freq_kind = 0;  // 0 List, 1 LinearSpaced, 2 LogSpaced
    std::vector<double> freq_values;
    double freq_start = 0, freq_end = 0;
    int64_t freq_number = 0;
    double sound_speed = 0, mass_density = 0;
    int problem_type = 1, method_type = 0, solver = 0;
    double tolerance = 0;
    int64_t max_iterations = 0;
    int64_t hm_leaf = 32;      // solve.rs:91-92, :119-120
    double hm_eta = 4.0;       // h_matrix.rs:136
    double hm_aca_tol = 1e-4;  // solve.rs:92, :120
    int incident_type = 0;
    double incident_vec[3] = {0, 0, 0};
    double incident_amp[2] = {0, 0};
    // every right-hand side: incident_wave first, then the optional
    // `additional_incident_waves` (the fields above hold the selected one)
    struct Wave {
        int type;
        double vec[3], amp[2];
    };
    std::vector<Wave> waves;
    int bc_type = 1;
    double bc_value[2] = {0, 0};
    int output_total = 0, output_pressure = 1;
    std::string output_file;
    std::vector<double> field_points;  // nfp x 3
};

struct Mesh {
    std::vector<double> nodes;  // 3 * nnodes
    std::vector<int64_t> body;
    std::vector<int32_t> etype;
    std::vector<int64_t> conn_off;
    std::vector<int64_t> conn;
    int64_t nbodies = 0;
    int64_t nelem() const { return (int64_t)body.size(); }
    int64_t nnodes() const { return (int64_t)nodes.size() / 3; }
};

UserInput parse_user_input(const std::string& json_text);
Mesh read_vtk(const std::string& path);
std::vector<double> frequency_list(const UserInput& in);

// ---------------------------------------------------------------------------
// Device buffer with grow-only capacity.
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    void ensure(size_t n) {
        if (n <= bytes) return;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        BEM_CUDA(cudaMalloc(&p, n));
        bytes = n;
    }
    template <class T> T* as() const { return static_cast<T*>(p); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    ~DevBuf() { release(); }
};

// Collocation geometry, structure of arrays on the device.  Every array is
// padded to `npad` (a multiple of 64) so that 64-point tiles can be copied into
// shared memory with 16-byte aligned bulk copies.
struct DevGeometry {
    int64_t n = 0, npad = 0;
    DevBuf buf;  // GEO_NARR arrays of npad doubles (see GeoArr)
    DevBuf buf32;  // GEO32_NARR arrays of npad floats (float-float coordinates, see Geo32Arr)
    double* arr(int k) const { return buf.as<double>() + (size_t)k * npad; }
    float* arr32(int k) const { return buf32.as<float>() + (size_t)k * npad; }
};

// x y z: collocation point; nx ny nz: unit normal as stored by the reference;
// ex ey ez: that normal normalised again (influence_matrix.rs:14-15 normalises
// per pair; the result only depends on the point); wa = wt * area.
enum GeoArr { GX = 0, GY, GZ, GNX, GNY, GNZ, GAREA, GWT, GWA, GEX, GEY, GEZ, GEO_NARR };
// Single-precision copy for the mixed form: coordinates split hi + lo.
// FP32 geometry: float-float coordinates, the unit normal as float-float
// (hi in FEX.., lo in FEXL..), and wt * area / (4 pi) as float-float (FWA,
// FWAL): a per-element rounding of that weight would scale the off-diagonal
// part of each column and not its diagonal, an error the solve amplifies.
enum Geo32Arr { FXH = 0, FXL, FYH, FYL, FZH, FZL, FEX, FEY, FEZ, FWA, FEXL, FEYL, FEZL, FWAL, GEO32_NARR };

struct Problem {
    UserInput in;
    Mesh mesh;
    std::vector<double> freqs;
    int64_t ifreq = 0;
    std::vector<double> cpts;  // host copy, n x 8
    int64_t n = 0, nfp = 0;
    DevGeometry geo;           // device collocation (computed by the collocation kernel)
    DevBuf d_fp;               // field points, 3 arrays of nfp_pad
    DevBuf d_fp32;             // field points as float-float, 6 arrays of nfp_pad
    int64_t nfp_pad = 0;
    int device = 0;
    int64_t nrhs() const { return in.waves.empty() ? 1 : (int64_t)in.waves.size(); }
    // makes right-hand side r the problem's incident wave
    void select_rhs(int64_t r) {
        if (in.waves.empty()) return;
        const UserInput::Wave& w = in.waves[(size_t)r];
        in.incident_type = w.type;
        for (int k = 0; k < 3; ++k) in.incident_vec[k] = w.vec[k];
        in.incident_amp[0] = w.amp[0];
        in.incident_amp[1] = w.amp[1];
    }
    double frequency() const { return freqs.empty() ? 0.0 : freqs[(size_t)ifreq]; }
    double omega() const { return 2.0 * 3.14159265358979323846 * frequency(); }
    double wavenumber() const { return omega() / in.sound_speed; }
};

// Per-stage timing recorded when profiling is enabled (CUDA events).
struct Stage {
    std::string name;
    double ms = 0;
    int64_t launches = 0;
    double bytes = 0;
};

struct LearnedNet;

// Launch parameters chosen by the offline sweep (cc_abstemious_gb300/tune.py
// writes tuning.json beside the library): per kernel, entries keyed by the
// problem size n and the number of systems; a lookup takes the nearest entry
// (log distance), else the built-in default.  Overrides (set through the C
// ABI, used by the sweep itself) take precedence.
struct TuneEntry {
    std::string kernel;
    int64_t n = 0, nsys = 0;
    std::vector<std::pair<std::string, int>> params;
};
struct TuningTable {
    std::vector<TuneEntry> entries;
    std::string source;  // file the table was read from ("" : built-in defaults)
    std::vector<std::pair<std::string, int>> overrides;  // "kernel.param" -> value
    int get(const char* kernel, const char* param, int64_t n, int64_t nsys, int dflt) const;
    int pick(const char* kernel, const char* param, int64_t n, int64_t nsys, int dflt) const {
        const std::string key = std::string(kernel) + "." + param;
        for (auto& kv : overrides)
            if (kv.first == key) return kv.second;
        return get(kernel, param, n, nsys, dflt);
    }
};
std::vector<TuneEntry> parse_tuning(const std::string& text);

struct Context {
    TuningTable tuning;
    int device = 0;
    bool profiling = false;
    std::shared_ptr<LearnedNet> net;  // preconditioner network (trained or loaded)
    std::vector<Stage> stages;
    void stage_add(const std::string& name, double ms, int64_t launches, double bytes) {
        for (auto& s : stages)
            if (s.name == name) {
                s.ms += ms;
                s.launches += launches;
                s.bytes += bytes;
                return;
            }
        stages.push_back({name, ms, launches, bytes});
    }
    cudaStream_t stream = nullptr;
    std::string last_error;
    int64_t launches = 0;
    // workspaces (grow-only)
    DevBuf w_mat, w_mat2, w_vec, w_small, w_flags, w_part, w_norm;
    // batched GMRES workspace and Krylov-preconditioned basis, LU factors,
    // diagonal-block inverses and panel workspace (grow-only, reused by
    // every mixed solve)
    DevBuf w_gm, w_gmz, w_lu_F, w_lu_D, w_lu_W, w_lu_P, w_lu_H;
    DevBuf w_upload;  // mesh staging of problem construction
    DevBuf w_piv;     // row pivots of the plain form's FP64 LU
    // results of the last bem_run
    std::vector<double> last_phi, last_vn;
    int64_t last_n = 0, last_nf = 0;
    void sync() { BEM_CUDA(cudaStreamSynchronize(stream)); }
};

// ---------------------------------------------------------------------------
// Host-side complex helpers.
struct cd { double re, im; };

// Kernel-side launch wrappers (defined in the .cu files).
void compute_collocation(Context& ctx, Problem& p);
void upload_field_points(Context& ctx, Problem& p);

// Problem scalars on the device.
struct KParams {
    double k;        // wavenumber
    double beta_im;  // BM coupling i/k -> imaginary part 1/k (0 for classical)
    int bm;          // Burton-Miller
    double hdiag;    // -0.5 exterior, 0 interior
    double gdiag_im; // BM: 0.5/k
};
KParams kparams(const Problem& p);
void lhs_factors(const Problem& p, cd& a, cd& b);
void rhs_factors(const Problem& p, cd& a, cd& b);

// Assembly (assembly.cu)
void assemble_surface_fp64(Context& ctx, const Problem& p, double2* H, double2* G, int64_t ld);
// A = alpha H + beta G and rowsum(gamma H + delta G) partials (fused solve path)
void assemble_system_fp64(Context& ctx, const Problem& p, double2* A, int64_t ld, cd alpha, cd beta,
                          cd gamma, cd delta, double2* rowsum /* n, may be null */);
// A_s = alpha_s H_s + beta_s G_s for several frequencies, split: the
// operator's FP32 rounding (float2, ld * n entries) followed by the FP32
// rounding of the remainder (`plane` = ld * n further on), evaluated in
// float-float (~2^-44 relative) with the geometry once per pair and
// e^{ik r} by recurrence for evenly spaced wavenumbers; systems 2 * plane
// float2 apart; norms[s] = ||A_s||_F.  remainder false: the FP32 roundings
// alone (the operator rounded once from its float-float value), systems
// `plane` float2 apart.
void assemble_system_split(Context& ctx, const Problem& p, const double* ks, const cd* alphas, const cd* betas,
                           int nsys, float2* A, int64_t ld, size_t plane, double* norms, bool remainder = true);
void assemble_system_fp32_body(Context& ctx, const Problem& p, const double* ks, const cd* alphas,
                               const cd* betas, const cd* gammas, const cd* deltas, int nsys, float2* A,
                               int64_t ld, size_t mat_stride, double2* rowsum, size_t vec_stride, double* norms);
// Several bodies, each with nsys frequencies (LHS operator only), in one
// launch; norms[g] = ||A_g||_F for the systems in body-major order.
struct BodyAsm32 {
    const Problem* p;
    int nsys;
    const double* ks;
    const cd *alphas, *betas;
    float2* A;  // system s at A + s * mat_stride
    int64_t ld;
    size_t mat_stride;
};
void assemble_fp32_multi(Context& ctx, const std::vector<BodyAsm32>& bodies, double* norms);
void evaluate_field32_batch(Context& ctx, const Problem& p, const double* ks, int nsys, const double2* phi,
                            const double2* vn, int64_t vstride, const double2* inc, double2* out);
void field_matrices_fp64(Context& ctx, const Problem& p, double2* M, double2* L, int64_t ld);
void evaluate_field(Context& ctx, const Problem& p, const double2* phi, const double2* vn,
                    const double2* inc, double2* out);
void row_or_column(Context& ctx, const Problem& p, const int64_t* dI, int64_t ni, const int64_t* dJ,
                   int64_t nj, int side, double2* out, int64_t diag_pos);
void incident_surface(Context& ctx, const Problem& p, double2* out);
// Incident values of several problems (frequency ifreq, incident wave rhs) in
// one launch: at the collocation points (field = false; with rhs_out, also the
// right-hand side sgn * inc + bc * rowsum) or at the field points.
struct IncItem {
    const Problem* p;
    int64_t ifreq, rhs;
    bool field;
    double2* out;
    double2* rhs_out;
    double sgn;
    cd bc;
    const double2* rowsum;
};
void incident_batch(Context& ctx, const std::vector<IncItem>& items);
void incident_field(Context& ctx, const Problem& p, double2* out);

// Dense linear algebra (dense.cu)
void lu_factor_fp64(Context& ctx, int64_t n, double2* A, int64_t lda, int32_t* d_piv, int* d_info);
void lu_solve_fp64(Context& ctx, int64_t n, const double2* A, int64_t lda, const int32_t* d_piv,
                   double2* b);
void gemv_fp64(Context& ctx, int64_t m, int64_t n, const double2* A, int64_t lda, const double2* x,
               double2* y, cd alpha, cd beta);
double frob_norm_fp64(Context& ctx, int64_t m, int64_t n, const double2* A, int64_t lda);

// GMRES (gmres.cu)
struct GmresResult {
    int64_t num_mv = 0, restarts = 0, iterations = 0;
    double error = 0;
    int flag = 0;
};
// Reference-faithful GMRES over a dense FP64 matrix (device), x in/out (device).
GmresResult gmres_dense_fp64(Context& ctx, int64_t n, const double2* A, int64_t lda, int64_t max_it,
                             double tol, double2* x);

}  // namespace bem

// Opaque handles of the C ABI.
struct bem_ctx {
    bem::Context c;
};
struct bem_problem {
    bem::Problem p;
};
