// C ABI of libbem_gb300.so (include/bem.h): context, problem (UserInput +
// PreData), the influence_matrix / incident_wave / solve / postprocess entry
// points and the analysis driver.
#include <dlfcn.h>
#include <chrono>
#include <cmath>
#include <cstring>
#include <fstream>
#include <memory>
#include <sstream>

#include "common.cuh"
#include "complex.cuh"
#include "gmres.cuh"
#include "hmatrix.cuh"
#include "mixed.cuh"
#include "precond.cuh"

namespace bem {

template <class F>
static bem_status guard(bem_ctx* ctx, F&& f) {
    try {
        f();
        return BEM_OK;
    } catch (const Error& e) {
        if (ctx) ctx->c.last_error = e.what();
        return e.status;
    } catch (const std::bad_alloc&) {
        if (ctx) ctx->c.last_error = "host allocation failed";
        return BEM_ERR_OOM;
    } catch (const std::exception& e) {
        if (ctx) ctx->c.last_error = e.what();
        return BEM_ERR_CUDA;
    }
}

static void set_device(Context& c) { BEM_CUDA(cudaSetDevice(c.device)); }

template <class T>
struct DevCopy {  // device view of a caller pointer (copies host data in/out)
    T* d = nullptr;
    DevBuf buf;
    const void* host = nullptr;
    size_t count = 0;
};

static void to_device(Context& c, DevBuf& b, const void* h, size_t bytes) {
    b.ensure(bytes ? bytes : 16);
    if (bytes) BEM_CUDA(cudaMemcpyAsync(b.p, h, bytes, cudaMemcpyHostToDevice, c.stream));
}
static void to_host(Context& c, void* h, const void* d, size_t bytes) {
    if (bytes) BEM_CUDA(cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, c.stream));
    c.sync();
}

static cd cmulh(cd a, cd b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }

// Uniform-BC right-hand side: rhs = s * rhs_inc + bc * rowsum (solve.rs:35-69).
__global__ void rhs_combine_kernel(int64_t n, double s, const double2* __restrict__ inc, z2 bc,
                                   const double2* __restrict__ rowsum, double2* __restrict__ out) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double2 v = cscale(inc[i], s);
    if (rowsum) cfma(v, bc, rowsum[i]);
    out[i] = v;
}

__global__ void fill_kernel(int64_t n, z2 v, double2* __restrict__ out) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = v;
}

__global__ void scale_kernel(int64_t n, z2 f, const double2* __restrict__ in, double2* __restrict__ out) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = cmul(f, in[i]);
}

void launch_rhs_combine(Context& c, int64_t n, double s, const double2* inc, cd bc, const double2* rowsum,
                        double2* out) {
    rhs_combine_kernel<<<(unsigned)((n + 255) / 256), 256, 0, c.stream>>>(n, s, inc, make_double2(bc.re, bc.im),
                                                                           rowsum, out);
    BEM_CHECK_LAUNCH(&c);
}
void launch_fill(Context& c, int64_t n, cd v, double2* out) {
    fill_kernel<<<(unsigned)((n + 255) / 256), 256, 0, c.stream>>>(n, make_double2(v.re, v.im), out);
    BEM_CHECK_LAUNCH(&c);
}
void launch_scale(Context& c, int64_t n, cd f, const double2* in, double2* out) {
    scale_kernel<<<(unsigned)((n + 255) / 256), 256, 0, c.stream>>>(n, make_double2(f.re, f.im), in, out);
    BEM_CHECK_LAUNCH(&c);
}

cd impedance_factor(const Problem& p) {
    // (0, -omega rho) / Z
    double zr = p.in.bc_value[0], zi = p.in.bc_value[1];
    double ni = -p.omega() * p.in.mass_density;
    double d = zr * zr + zi * zi;
    return {(ni * zi) / d, (ni * zr) / d};
}

// Unpack the solved vector into (phi, vn) by boundary condition (solve.rs:35-69).
void unpack_solution(Context& c, const Problem& p, const double2* x, double2* phi, double2* vn) {
    int64_t n = p.n;
    cd bcv = {p.in.bc_value[0], p.in.bc_value[1]};
    if (p.in.bc_type == 0) {
        launch_fill(c, n, bcv, phi);
        BEM_CUDA(cudaMemcpyAsync(vn, x, sizeof(double2) * n, cudaMemcpyDeviceToDevice, c.stream));
    } else if (p.in.bc_type == 1) {
        launch_fill(c, n, bcv, vn);
        BEM_CUDA(cudaMemcpyAsync(phi, x, sizeof(double2) * n, cudaMemcpyDeviceToDevice, c.stream));
    } else {
        BEM_CUDA(cudaMemcpyAsync(phi, x, sizeof(double2) * n, cudaMemcpyDeviceToDevice, c.stream));
        launch_scale(c, n, impedance_factor(p), x, vn);
    }
}

// unpack_solution for several systems in one launch.
struct UnpackJob {
    int64_t n, blk0;
    int bc_type, pad;
    double2 bcv, f;  // boundary value; impedance factor
    const double2* x;
    double2 *phi, *vn;
};

__global__ void unpack_batch_kernel(const UnpackJob* __restrict__ jobs, int njobs) {
    const int64_t b = blockIdx.x;
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (jobs[mid].blk0 <= b) lo = mid;
        else hi = mid - 1;
    }
    const UnpackJob& J = jobs[lo];
    const int64_t i = (b - J.blk0) * 256 + threadIdx.x;
    if (i >= J.n) return;
    const double2 x = J.x[i];
    if (J.bc_type == 0) {
        J.phi[i] = J.bcv;
        J.vn[i] = x;
    } else if (J.bc_type == 1) {
        J.phi[i] = x;
        J.vn[i] = J.bcv;
    } else {
        J.phi[i] = x;
        J.vn[i] = cmul(J.f, x);
    }
}

void unpack_batch(Context& c, const std::vector<UnpackItem>& items) {
    std::vector<UnpackJob> jobs;
    int64_t blk = 0;
    for (const UnpackItem& it : items) {
        Problem& p = const_cast<Problem&>(*it.p);
        const int64_t f0 = p.ifreq;
        p.ifreq = it.ifreq;
        UnpackJob J{};
        J.n = p.n;
        J.blk0 = blk;
        J.bc_type = p.in.bc_type;
        J.bcv = make_double2(p.in.bc_value[0], p.in.bc_value[1]);
        if (p.in.bc_type == 2) {
            const cd f = impedance_factor(p);
            J.f = make_double2(f.re, f.im);
        }
        p.ifreq = f0;
        J.x = it.x;
        J.phi = it.phi;
        J.vn = it.vn;
        blk += (J.n + 255) / 256;
        jobs.push_back(J);
    }
    if (jobs.empty()) return;
    DevBuf d;
    d.ensure(sizeof(UnpackJob) * jobs.size());
    BEM_CUDA(cudaMemcpyAsync(d.p, jobs.data(), sizeof(UnpackJob) * jobs.size(), cudaMemcpyHostToDevice, c.stream));
    unpack_batch_kernel<<<(unsigned)blk, 256, 0, c.stream>>>(d.as<UnpackJob>(), (int)jobs.size());
    BEM_CHECK_LAUNCH(&c);
    c.sync();  // the job list is freed on return
}

// Dense plain-FP64 surface solve on device vectors (solve.rs:24-71 and
// :153-171): the fused kernel assembles the system matrix alpha H + beta G and
// the uniform-BC right-hand side in one pass.
// reuse_lu (Direct solver only): the previous call factored this frequency's
// operator into the context's buffers (w_mat, w_piv, and the boundary
// condition's row sums in w_vec); only the right-hand side is new (several
// incident waves share one factorization).
void solve_surface_dense_fp64(Context& c, const Problem& p, const double2* d_rhs_inc, double2* d_phi,
                              double2* d_vn, bem_solve_report* rep, double2* d_A_keep, bool reuse_lu) {
    int64_t n = p.n;
    cd a, b, g, d;
    lhs_factors(p, a, b);
    rhs_factors(p, g, d);
    bool need_rowsum = !(p.in.bc_value[0] == 0.0 && p.in.bc_value[1] == 0.0) && p.in.bc_type != 2;
    reuse_lu = reuse_lu && p.in.solver == 0 && !d_A_keep;
    double2* A = d_A_keep;
    if (!A) {
        if (!reuse_lu) c.w_mat.ensure(sizeof(double2) * (size_t)n * n);
        A = c.w_mat.as<double2>();
    }
    if (!reuse_lu) c.w_vec.ensure(sizeof(double2) * (size_t)n * 4);
    double2* rowsum = c.w_vec.as<double2>();
    double2* x = rowsum + n;
    if (!reuse_lu) assemble_system_fp64(c, p, A, n, a, b, g, d, need_rowsum ? rowsum : nullptr);
    double s = p.in.bc_type == 0 ? 1.0 : -1.0;
    launch_rhs_combine(c, n, s, d_rhs_inc, {p.in.bc_value[0], p.in.bc_value[1]}, need_rowsum ? rowsum : nullptr, x);
    if (p.in.solver == 0) {
        c.w_flags.ensure(256);
        if (!reuse_lu) {
            c.w_piv.ensure(sizeof(int32_t) * (size_t)n);
            lu_factor_fp64(c, n, A, n, c.w_piv.as<int32_t>(), c.w_flags.as<int>() + 1);
        }
        lu_solve_fp64(c, n, A, n, c.w_piv.as<int32_t>(), x);
        int info = 0;
        to_host(c, &info, c.w_flags.as<int>() + 1, sizeof(int));
        if (rep) rep->flag = 3;
        require(info == 0, "LU factorisation found a zero pivot (column " + std::to_string(info) + ")",
                BEM_ERR_SINGULAR);
    } else {
        GmresResult r = gmres_dense_fp64(c, n, A, n, p.in.max_iterations, p.in.tolerance, x);
        if (rep) {
            rep->num_mv = r.num_mv;
            rep->restarts = r.restarts;
            rep->iterations = r.iterations;
            rep->backward_error = r.error;
            rep->flag = r.flag;
        }
    }
    unpack_solution(c, p, x, d_phi, d_vn);
}

void solve_surface_fp64(Context& c, const Problem& p, const double2* d_rhs_inc, double2* d_phi, double2* d_vn,
                        bem_solve_report* rep) {
    if (p.in.solver == 2) solve_surface_hmatrix(c, p, d_rhs_inc, d_phi, d_vn, rep);
    else solve_surface_dense_fp64(c, p, d_rhs_inc, d_phi, d_vn, rep, nullptr, false);
}

// The built-in launch parameters (used where no tuning entry applies).
int tuning_default(const std::string& kernel, const std::string& param) {
    if (kernel == "lu_gemm_trail") return param == "sb_r" ? 8 : param == "sb_c" ? 32 : -1;
    if (kernel == "gm_apply_fp32" && param == "unroll") return 8;
    if (kernel == "assemble32" && param == "min_ctas") return 3;
    return -1;
}

// tuning.json in the directory of this library.
static std::string default_tuning_path() {
    Dl_info info;
    if (!dladdr(reinterpret_cast<void*>(&tuning_default), &info) || !info.dli_fname) return "";
    std::string so = info.dli_fname;
    const size_t slash = so.rfind('/');
    const std::string dir = slash == std::string::npos ? "." : so.substr(0, slash);
    const std::string path = dir + "/tuning.json";
    std::ifstream f(path);
    return f.good() ? path : "";
}

// Reads a tuning table; a missing file is an error only when it was asked for.
static void load_tuning_file(Context& c, const std::string& path, bool required) {
    std::ifstream f(path);
    if (!f.good()) {
        require(!required, "cannot open tuning table " + path);
        return;
    }
    std::stringstream ss;
    ss << f.rdbuf();
    c.tuning.entries = parse_tuning(ss.str());
    c.tuning.source = path;
}

static void load_problem(Context& c, Problem& p, const std::string& json, const std::string& base_dir) {
    p.in = parse_user_input(json);
    std::string path = p.in.mesh_file;
    if (!base_dir.empty() && !path.empty() && path[0] != '/') path = base_dir + "/" + path;
    p.mesh = read_vtk(path);
    p.freqs = frequency_list(p.in);
    p.ifreq = 0;
    p.device = c.device;
    compute_collocation(c, p);
    upload_field_points(c, p);
    c.sync();
}

}  // namespace bem

using namespace bem;

extern "C" {

BEM_API const char* bem_version(void) { return "bem_gb300 1.0 (sm_103a)"; }

BEM_API bem_status bem_ctx_create(int device, bem_ctx** out) {
    if (!out) return BEM_ERR_BAD_INPUT;
    *out = nullptr;
    std::unique_ptr<bem_ctx> ctx(new bem_ctx());
    bem_status st = guard(nullptr, [&] {
        int count = 0;
        BEM_CUDA(cudaGetDeviceCount(&count));
        require(device >= 0 && device < count, "no CUDA device " + std::to_string(device));
        ctx->c.device = device;
        set_device(ctx->c);
        BEM_CUDA(cudaStreamCreateWithFlags(&ctx->c.stream, cudaStreamNonBlocking));
        // the tuned launch table: BEM_TUNING_FILE ("none": built-in
        // defaults), else tuning.json beside the library when present
        const char* env = std::getenv("BEM_TUNING_FILE");
        std::string path = env ? env : default_tuning_path();
        if (!path.empty() && path != "none") load_tuning_file(ctx->c, path, env != nullptr);
    });
    if (st == BEM_OK) *out = ctx.release();
    return st;
}

BEM_API bem_status bem_ctx_load_tuning(bem_ctx* ctx, const char* path) {
    if (!ctx) return BEM_ERR_BAD_INPUT;
    return guard(ctx, [&] {
        if (!path) {
            ctx->c.tuning.entries.clear();
            ctx->c.tuning.source.clear();
            return;
        }
        load_tuning_file(ctx->c, path, true);
    });
}

BEM_API bem_status bem_ctx_set_tuning(bem_ctx* ctx, const char* kernel, const char* param, int value) {
    if (!ctx || !kernel || !param) return BEM_ERR_BAD_INPUT;
    auto& ov = ctx->c.tuning.overrides;
    const std::string key = std::string(kernel) + "." + param;
    for (size_t i = 0; i < ov.size(); ++i)
        if (ov[i].first == key) {
            ov.erase(ov.begin() + (long)i);
            break;
        }
    if (value >= 0) ov.emplace_back(key, value);
    return BEM_OK;
}

BEM_API int bem_ctx_get_tuning(const bem_ctx* ctx, const char* kernel, const char* param, int64_t n, int64_t nsys) {
    if (!ctx || !kernel || !param) return -1;
    // the LU step-group size: the rule of lu_group (8 from 12000 unknowns on)
    if (std::string(kernel) == "lu_gemm_trail" && std::string(param) == "group") return lu_group(ctx->c, n, nsys);
    return ctx->c.tuning.pick(kernel, param, n, nsys, tuning_default(kernel, param));
}

BEM_API const char* bem_ctx_tuning_source(const bem_ctx* ctx) { return ctx ? ctx->c.tuning.source.c_str() : ""; }

BEM_API void bem_ctx_destroy(bem_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->c.device);
    if (ctx->c.stream) {
        cudaStreamSynchronize(ctx->c.stream);
        cudaStreamDestroy(ctx->c.stream);
    }
    delete ctx;
}

BEM_API const char* bem_last_error(const bem_ctx* ctx) { return ctx ? ctx->c.last_error.c_str() : ""; }
BEM_API int64_t bem_ctx_kernel_launches(const bem_ctx* ctx) { return ctx ? ctx->c.launches : 0; }

BEM_API bem_status bem_ctx_set_profiling(bem_ctx* ctx, int on) {
    if (!ctx) return BEM_ERR_BAD_INPUT;
    ctx->c.profiling = on != 0;
    return BEM_OK;
}

BEM_API void* bem_ctx_stream(const bem_ctx* ctx) { return ctx ? (void*)ctx->c.stream : nullptr; }

BEM_API int64_t bem_ctx_profile_count(const bem_ctx* ctx) { return ctx ? (int64_t)ctx->c.stages.size() : 0; }

BEM_API bem_status bem_ctx_profile_get(const bem_ctx* ctx, int64_t i, char* name, int64_t name_len, double* ms,
                                       int64_t* launches, double* bytes) {
    if (!ctx || i < 0 || i >= (int64_t)ctx->c.stages.size()) return BEM_ERR_BAD_INPUT;
    const Stage& s = ctx->c.stages[(size_t)i];
    if (name && name_len > 0) {
        std::strncpy(name, s.name.c_str(), (size_t)name_len - 1);
        name[name_len - 1] = 0;
    }
    if (ms) *ms = s.ms;
    if (launches) *launches = s.launches;
    if (bytes) *bytes = s.bytes;
    return BEM_OK;
}

BEM_API bem_status bem_problem_from_json(bem_ctx* ctx, const char* json, const char* base_dir, bem_problem** out) {
    if (!ctx || !json || !out) return BEM_ERR_BAD_INPUT;
    *out = nullptr;
    std::unique_ptr<bem_problem> p(new bem_problem());
    bem_status st = guard(ctx, [&] {
        set_device(ctx->c);
        load_problem(ctx->c, p->p, json, base_dir ? base_dir : "");
    });
    if (st == BEM_OK) *out = p.release();
    return st;
}

BEM_API bem_status bem_problem_from_file(bem_ctx* ctx, const char* path, bem_problem** out) {
    if (!ctx || !path || !out) return BEM_ERR_BAD_INPUT;
    std::string text;
    bem_status st = guard(ctx, [&] {
        std::ifstream f(path);
        require(f.good(), std::string("cannot open input file ") + path);
        std::stringstream ss;
        ss << f.rdbuf();
        text = ss.str();
    });
    if (st != BEM_OK) return st;
    // mesh_file is resolved against the working directory like the reference
    return bem_problem_from_json(ctx, text.c_str(), nullptr, out);
}

BEM_API void bem_problem_destroy(bem_problem* p) {
    if (!p) return;
    cudaSetDevice(p->p.device);
    delete p;
}

BEM_API bem_status bem_problem_get_info(const bem_problem* pp, bem_problem_info* o) {
    if (!pp || !o) return BEM_ERR_BAD_INPUT;
    const Problem& p = pp->p;
    std::memset(o, 0, sizeof *o);
    o->sound_speed = p.in.sound_speed;
    o->mass_density = p.in.mass_density;
    o->problem_type = p.in.problem_type;
    o->method_type = p.in.method_type;
    o->solver = p.in.solver;
    o->incident_type = p.in.incident_type;
    o->bc_type = p.in.bc_type;
    o->output_total = p.in.output_total;
    o->output_pressure = p.in.output_pressure;
    o->body_index = (int32_t)p.in.body_index;
    o->tolerance = p.in.tolerance;
    o->max_iterations = p.in.max_iterations;
    for (int k = 0; k < 3; ++k) o->incident_vec[k] = p.in.incident_vec[k];
    for (int k = 0; k < 2; ++k) { o->incident_amp[k] = p.in.incident_amp[k]; o->bc_value[k] = p.in.bc_value[k]; }
    o->hm_leaf = p.in.hm_leaf;
    o->hm_eta = p.in.hm_eta;
    o->hm_aca_tol = p.in.hm_aca_tol;
    o->num_eqn = p.n;
    o->num_field_points = p.nfp;
    o->num_frequencies = (int64_t)p.freqs.size();
    o->mesh_elements = p.mesh.nelem();
    o->mesh_nodes = p.mesh.nnodes();
    o->mesh_bodies = p.mesh.nbodies;
    o->num_rhs = p.nrhs();
    return BEM_OK;
}

BEM_API bem_status bem_problem_frequencies(const bem_problem* p, double* out) {
    if (!p || !out) return BEM_ERR_BAD_INPUT;
    std::memcpy(out, p->p.freqs.data(), sizeof(double) * p->p.freqs.size());
    return BEM_OK;
}

BEM_API bem_status bem_problem_set_frequency_index(bem_problem* p, int64_t index) {
    if (!p || index < 0 || index >= (int64_t)p->p.freqs.size()) return BEM_ERR_BAD_INPUT;
    p->p.ifreq = index;
    return BEM_OK;
}

BEM_API bem_status bem_collocation(bem_ctx* ctx, const bem_problem* p, double* out) {
    if (!ctx || !p || !out) return BEM_ERR_BAD_INPUT;
    std::memcpy(out, p->p.cpts.data(), sizeof(double) * p->p.cpts.size());
    return BEM_OK;
}

BEM_API bem_status bem_get_dense_surface_matrices(bem_ctx* ctx, const bem_problem* pp, bem_cplx* H, bem_cplx* G,
                                                  int64_t ld, bem_mem mem) {
    if (!ctx || !pp || !H || !G) return BEM_ERR_BAD_INPUT;
    return guard(ctx, [&] {
        Context& c = ctx->c;
        const Problem& p = pp->p;
        set_device(c);
        require(ld >= p.n, "ld < n");
        if (mem == BEM_MEM_DEVICE) {
            assemble_surface_fp64(c, p, reinterpret_cast<double2*>(H), reinterpret_cast<double2*>(G), ld);
            c.sync();
            return;
        }
        size_t bytes = sizeof(double2) * (size_t)p.n * p.n;
        c.w_mat.ensure(bytes);
        c.w_mat2.ensure(bytes);
        assemble_surface_fp64(c, p, c.w_mat.as<double2>(), c.w_mat2.as<double2>(), p.n);
        BEM_CUDA(cudaMemcpy2DAsync(H, sizeof(double2) * ld, c.w_mat.p, sizeof(double2) * p.n, sizeof(double2) * p.n,
                                   p.n, cudaMemcpyDeviceToHost, c.stream));
        BEM_CUDA(cudaMemcpy2DAsync(G, sizeof(double2) * ld, c.w_mat2.p, sizeof(double2) * p.n, sizeof(double2) * p.n,
                                   p.n, cudaMemcpyDeviceToHost, c.stream));
        c.sync();
    });
}

BEM_API bem_status bem_assemble_operator(bem_ctx* ctx, const bem_problem* pp, int kind, int64_t f0, int64_t nf,
                                         bem_cplx* A, int64_t lda) {
    if (!ctx || !pp || !A || kind < 0 || kind > 2) return BEM_ERR_BAD_INPUT;
    return guard(ctx, [&] {
        Context& c = ctx->c;
        Problem& p = const_cast<Problem&>(pp->p);
        set_device(c);
        const int64_t n = p.n, ld = p.geo.npad, NF = (int64_t)p.freqs.size();
        require(lda >= n, "lda < n");
        require(f0 >= 0 && nf >= 1 && f0 + nf <= NF, "frequency range outside the problem's list");
        const int64_t saved = p.ifreq;
        std::vector<double> ks((size_t)nf);
        std::vector<cd> al((size_t)nf), be((size_t)nf), ga((size_t)nf), de((size_t)nf);
        for (int64_t f = 0; f < nf; ++f) {
            p.ifreq = f0 + f;
            ks[(size_t)f] = p.wavenumber();
            lhs_factors(p, al[(size_t)f], be[(size_t)f]);
            rhs_factors(p, ga[(size_t)f], de[(size_t)f]);
        }
        p.ifreq = saved;
        const size_t plane = (size_t)ld * n;
        DevBuf d, norms;
        const bool two = kind == 1;  // the split store has a remainder plane
        d.ensure(sizeof(float2) * plane * (two ? 2 : 1) * (size_t)nf);
        norms.ensure(sizeof(double) * (size_t)nf);
        if (kind == 0)
            assemble_system_fp32_body(c, p, ks.data(), al.data(), be.data(), ga.data(), de.data(), (int)nf,
                                      d.as<float2>(), ld, plane, nullptr, 0, norms.as<double>());
        else
            assemble_system_split(c, p, ks.data(), al.data(), be.data(), (int)nf, d.as<float2>(), ld, plane,
                                  norms.as<double>(), two);
        std::vector<float2> h(plane * (two ? 2 : 1) * (size_t)nf);
        BEM_CUDA(cudaMemcpyAsync(h.data(), d.p, sizeof(float2) * h.size(), cudaMemcpyDeviceToHost, c.stream));
        c.sync();
        const size_t sstride = plane * (two ? 2 : 1);
        for (int64_t f = 0; f < nf; ++f)
            for (int64_t j = 0; j < n; ++j)
                for (int64_t i = 0; i < n; ++i) {
                    const size_t o = (size_t)f * sstride + (size_t)j * ld + i;
                    double re = h[o].x, im = h[o].y;
                    if (two) {
                        re += (double)h[o + plane].x;
                        im += (double)h[o + plane].y;
                    }
                    A[(size_t)f * lda * n + (size_t)j * lda + i] = bem_cplx{re, im};
                }
    });
}

BEM_API bem_status bem_get_dense_field_matrices(bem_ctx* ctx, const bem_problem* pp, bem_cplx* M, bem_cplx* L,
                                                int64_t ld, bem_mem mem) {
    if (!ctx || !pp || !M || !L) return BEM_ERR_BAD_INPUT;
    return guard(ctx, [&] {
        Context& c = ctx->c;
        const Problem& p = pp->p;
        set_device(c);
        require(ld >= p.nfp && ld >= 1, "ld < number of field points");
        if (p.nfp == 0) return;
        if (mem == BEM_MEM_DEVICE) {
            field_matrices_fp64(c, p, reinterpret_cast<double2*>(M), reinterpret_cast<double2*>(L), ld);
            c.sync();
            return;
        }
        size_t bytes = sizeof(double2) * (size_t)p.nfp * p.n;
        c.w_mat.ensure(bytes);
        c.w_mat2.ensure(bytes);
        field_matrices_fp64(c, p, c.w_mat.as<double2>(), c.w_mat2.as<double2>(), p.nfp);
        BEM_CUDA(cudaMemcpy2DAsync(M, sizeof(double2) * ld, c.w_mat.p, sizeof(double2) * p.nfp,
                                   sizeof(double2) * p.nfp, p.n, cudaMemcpyDeviceToHost, c.stream));
        BEM_CUDA(cudaMemcpy2DAsync(L, sizeof(double2) * ld, c.w_mat2.p, sizeof(double2) * p.nfp,
                                   sizeof(double2) * p.nfp, p.n, cudaMemcpyDeviceToHost, c.stream));
        c.sync();
    });
}

BEM_API bem_status bem_get_surface_row_or_column(bem_ctx* ctx, const bem_problem* pp, const int64_t* I, int64_t ni,
                                                 const int64_t* J, int64_t nj, bem_side side, bem_cplx* out) {
    if (!ctx || !pp || !out || (ni && !I) || (nj && !J)) return BEM_ERR_BAD_INPUT;
    return guard(ctx, [&] {
        Context& c = ctx->c;
        const Problem& p = pp->p;
        set_device(c);
        require((ni == 1) != (nj == 1), "Invalid call to get_surface_row_or_column: i or j must be singleton");
        for (int64_t t = 0; t < ni; ++t) require(I[t] >= 0 && I[t] < p.n, "row index out of range");
        for (int64_t t = 0; t < nj; ++t) require(J[t] >= 0 && J[t] < p.n, "column index out of range");
        int64_t len = ni == 1 ? nj : ni;
        int64_t diag = -1;
        for (int64_t t = 0; t < len && diag < 0; ++t) {
            int64_t i = ni == 1 ? I[0] : I[t], j = ni == 1 ? J[t] : J[0];
            if (i == j) diag = t;
        }
        DevBuf dI, dJ, dout;
        to_device(c, dI, I, sizeof(int64_t) * ni);
        to_device(c, dJ, J, sizeof(int64_t) * nj);
        dout.ensure(sizeof(double2) * (len ? len : 1));
        row_or_column(c, p, dI.as<int64_t>(), ni, dJ.as<int64_t>(), nj, side == BEM_SIDE_LHS ? 1 : 0,
                      dout.as<double2>(), diag);
        to_host(c, out, dout.p, sizeof(double2) * len);
    });
}

BEM_API bem_status bem_get_system_matrix_fp32(bem_ctx* ctx, const bem_problem* pp, float* A, int64_t ld) {
    if (!ctx || !pp || !A) return BEM_ERR_BAD_INPUT;
    return guard(ctx, [&] {
        Context& c = ctx->c;
        const Problem& p = pp->p;
        set_device(c);
        require(ld >= p.n, "ld < n");
        cd a, b, g, d;
        lhs_factors(p, a, b);
        rhs_factors(p, g, d);
        double k = p.wavenumber();
        const int64_t ldd = p.geo.npad;
        DevBuf m, nrm;
        m.ensure(sizeof(float2) * (size_t)ldd * p.n);
        nrm.ensure(sizeof(double));
        assemble_system_fp32_body(c, p, &k, &a, &b, &g, &d, 1, m.as<float2>(), ldd, (size_t)ldd * p.n, nullptr, 0,
                                  nrm.as<double>());
        BEM_CUDA(cudaMemcpy2DAsync(A, sizeof(float2) * ld, m.p, sizeof(float2) * ldd, sizeof(float2) * p.n, p.n,
                                   cudaMemcpyDeviceToHost, c.stream));
        c.sync();
    });
}

BEM_API bem_status bem_get_incident_surface(bem_ctx* ctx, const bem_problem* pp, bem_cplx* rhs_inc) {
    if (!ctx || !pp || !rhs_inc) return BEM_ERR_BAD_INPUT;
    return guard(ctx, [&] {
        Context& c = ctx->c;
        set_device(c);
        DevBuf d;
        d.ensure(sizeof(double2) * pp->p.n);
        incident_surface(c, pp->p, d.as<double2>());
        to_host(c, rhs_inc, d.p, sizeof(double2) * pp->p.n);
    });
}

BEM_API bem_status bem_get_incident_field(bem_ctx* ctx, const bem_problem* pp, bem_cplx* out) {
    if (!ctx || !pp || (!out && pp->p.nfp)) return BEM_ERR_BAD_INPUT;
    return guard(ctx, [&] {
        Context& c = ctx->c;
        set_device(c);
        if (pp->p.nfp == 0) return;
        DevBuf d;
        d.ensure(sizeof(double2) * pp->p.nfp);
        incident_field(c, pp->p, d.as<double2>());
        to_host(c, out, d.p, sizeof(double2) * pp->p.nfp);
    });
}

BEM_API bem_status bem_solve_for_surface(bem_ctx* ctx, const bem_problem* pp, const bem_cplx* rhs_inc, bem_cplx* phi,
                                         bem_cplx* vn, bem_solve_report* rep) {
    if (!ctx || !pp || !rhs_inc || !phi || !vn) return BEM_ERR_BAD_INPUT;
    if (rep) { std::memset(rep, 0, sizeof *rep); rep->rel_err_vs_lu = -1; }
    auto t0 = std::chrono::steady_clock::now();
    bem_status st = guard(ctx, [&] {
        Context& c = ctx->c;
        const Problem& p = pp->p;
        set_device(c);
        DevBuf d;
        d.ensure(sizeof(double2) * p.n * 3);
        double2* dr = d.as<double2>();
        BEM_CUDA(cudaMemcpyAsync(dr, rhs_inc, sizeof(double2) * p.n, cudaMemcpyHostToDevice, c.stream));
        solve_surface_fp64(c, p, dr, dr + p.n, dr + 2 * p.n, rep);
        BEM_CUDA(cudaMemcpyAsync(phi, dr + p.n, sizeof(double2) * p.n, cudaMemcpyDeviceToHost, c.stream));
        BEM_CUDA(cudaMemcpyAsync(vn, dr + 2 * p.n, sizeof(double2) * p.n, cudaMemcpyDeviceToHost, c.stream));
        c.sync();
    });
    if (rep) rep->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (st == BEM_OK && rep && rep->flag == 2) return BEM_ERR_NOT_CONVERGED;
    return st;
}

BEM_API bem_status bem_solve_lu(bem_ctx* ctx, int64_t n, const bem_cplx* A, int64_t lda, bem_cplx* x, bem_mem mem) {
    if (!ctx || !A || !x || n < 0 || lda < n) return BEM_ERR_BAD_INPUT;
    return guard(ctx, [&] {
        Context& c = ctx->c;
        set_device(c);
        if (n == 0) return;
        c.w_mat.ensure(sizeof(double2) * (size_t)n * n);
        double2* W = c.w_mat.as<double2>();
        BEM_CUDA(cudaMemcpy2DAsync(W, sizeof(double2) * n, A, sizeof(double2) * lda, sizeof(double2) * n, n,
                                   mem == BEM_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                   c.stream));
        DevBuf piv, xb;
        piv.ensure(sizeof(int32_t) * n);
        double2* dx;
        if (mem == BEM_MEM_DEVICE) dx = reinterpret_cast<double2*>(x);
        else {
            to_device(c, xb, x, sizeof(double2) * n);
            dx = xb.as<double2>();
        }
        c.w_flags.ensure(256);
        lu_factor_fp64(c, n, W, n, piv.as<int32_t>(), c.w_flags.as<int>() + 1);
        lu_solve_fp64(c, n, W, n, piv.as<int32_t>(), dx);
        int info = 0;
        to_host(c, &info, c.w_flags.as<int>() + 1, sizeof(int));
        if (mem == BEM_MEM_HOST) to_host(c, x, dx, sizeof(double2) * n);
        require(info == 0, "LU factorisation found a zero pivot (column " + std::to_string(info) + ")",
                BEM_ERR_SINGULAR);
    });
}

BEM_API bem_status bem_gmres_solve(bem_ctx* ctx, int64_t n, const bem_cplx* A, int64_t lda, int64_t max_it,
                                   double tol, bem_cplx* x, bem_solve_report* rep, bem_mem mem) {
    if (!ctx || !A || !x || n <= 0 || lda < n) return BEM_ERR_BAD_INPUT;
    if (rep) { std::memset(rep, 0, sizeof *rep); rep->rel_err_vs_lu = -1; }
    GmresResult r;
    auto t0 = std::chrono::steady_clock::now();
    bem_status st = guard(ctx, [&] {
        Context& c = ctx->c;
        set_device(c);
        const double2* dA = reinterpret_cast<const double2*>(A);
        int64_t ldd = lda;
        if (mem == BEM_MEM_HOST) {
            c.w_mat.ensure(sizeof(double2) * (size_t)n * n);
            BEM_CUDA(cudaMemcpy2DAsync(c.w_mat.p, sizeof(double2) * n, A, sizeof(double2) * lda, sizeof(double2) * n,
                                       n, cudaMemcpyHostToDevice, c.stream));
            dA = c.w_mat.as<double2>();
            ldd = n;
        }
        DevBuf xb;
        double2* dx;
        if (mem == BEM_MEM_DEVICE) dx = reinterpret_cast<double2*>(x);
        else {
            to_device(c, xb, x, sizeof(double2) * n);
            dx = xb.as<double2>();
        }
        r = gmres_dense_fp64(c, n, dA, ldd, max_it, tol, dx);
        if (mem == BEM_MEM_HOST) to_host(c, x, dx, sizeof(double2) * n);
    });
    if (rep && st == BEM_OK) {
        rep->num_mv = r.num_mv;
        rep->restarts = r.restarts;
        rep->iterations = r.iterations;
        rep->backward_error = r.error;
        rep->flag = r.flag;
        rep->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    if (st == BEM_OK && r.flag == 2) return BEM_ERR_NOT_CONVERGED;
    return st;
}

BEM_API bem_status bem_get_field(bem_ctx* ctx, const bem_problem* pp, const bem_cplx* M, const bem_cplx* L, int64_t ld,
                                 const bem_cplx* phi, const bem_cplx* vn, const bem_cplx* inc, bem_cplx* out,
                                 bem_mem mem) {
    if (!ctx || !pp || !M || !L || !phi || !vn || !inc || !out) return BEM_ERR_BAD_INPUT;
    return guard(ctx, [&] {
        Context& c = ctx->c;
        const Problem& p = pp->p;
        set_device(c);
        int64_t nfp = p.nfp, n = p.n;
        if (nfp == 0) return;
        require(ld >= nfp, "ld < number of field points");
        const double2 *dM, *dL, *dphi, *dvn, *dinc;
        double2* dout;
        DevBuf bm, bl, bv;
        if (mem == BEM_MEM_DEVICE) {
            dM = reinterpret_cast<const double2*>(M);
            dL = reinterpret_cast<const double2*>(L);
            dphi = reinterpret_cast<const double2*>(phi);
            dvn = reinterpret_cast<const double2*>(vn);
            dinc = reinterpret_cast<const double2*>(inc);
            dout = reinterpret_cast<double2*>(out);
        } else {
            bm.ensure(sizeof(double2) * (size_t)ld * n);
            bl.ensure(sizeof(double2) * (size_t)ld * n);
            BEM_CUDA(cudaMemcpyAsync(bm.p, M, sizeof(double2) * (size_t)ld * n, cudaMemcpyHostToDevice, c.stream));
            BEM_CUDA(cudaMemcpyAsync(bl.p, L, sizeof(double2) * (size_t)ld * n, cudaMemcpyHostToDevice, c.stream));
            bv.ensure(sizeof(double2) * (2 * n + 2 * nfp));
            double2* v = bv.as<double2>();
            BEM_CUDA(cudaMemcpyAsync(v, phi, sizeof(double2) * n, cudaMemcpyHostToDevice, c.stream));
            BEM_CUDA(cudaMemcpyAsync(v + n, vn, sizeof(double2) * n, cudaMemcpyHostToDevice, c.stream));
            BEM_CUDA(cudaMemcpyAsync(v + 2 * n, inc, sizeof(double2) * nfp, cudaMemcpyHostToDevice, c.stream));
            dM = bm.as<double2>();
            dL = bl.as<double2>();
            dphi = v;
            dvn = v + n;
            dinc = v + 2 * n;
            dout = v + 2 * n + nfp;
        }
        // out = [inc] - M phi + L vn   (solve.rs:173-185)
        if (p.in.output_total)
            BEM_CUDA(cudaMemcpyAsync(dout, dinc, sizeof(double2) * nfp, cudaMemcpyDeviceToDevice, c.stream));
        gemv_fp64(c, nfp, n, dM, ld, dphi, dout, {-1.0, 0.0}, p.in.output_total ? cd{1.0, 0.0} : cd{0.0, 0.0});
        gemv_fp64(c, nfp, n, dL, ld, dvn, dout, {1.0, 0.0}, {1.0, 0.0});
        if (mem == BEM_MEM_HOST) to_host(c, out, dout, sizeof(double2) * nfp);
        else c.sync();
    });
}

BEM_API bem_status bem_evaluate_field(bem_ctx* ctx, const bem_problem* pp, const bem_cplx* phi, const bem_cplx* vn,
                                      const bem_cplx* inc, bem_cplx* out) {
    if (!ctx || !pp || !phi || !vn || !out) return BEM_ERR_BAD_INPUT;
    return guard(ctx, [&] {
        Context& c = ctx->c;
        const Problem& p = pp->p;
        set_device(c);
        if (p.nfp == 0) return;
        DevBuf b;
        b.ensure(sizeof(double2) * (2 * p.n + 2 * p.nfp));
        double2* v = b.as<double2>();
        BEM_CUDA(cudaMemcpyAsync(v, phi, sizeof(double2) * p.n, cudaMemcpyHostToDevice, c.stream));
        BEM_CUDA(cudaMemcpyAsync(v + p.n, vn, sizeof(double2) * p.n, cudaMemcpyHostToDevice, c.stream));
        const double2* dinc = nullptr;
        if (p.in.output_total && inc) {
            BEM_CUDA(cudaMemcpyAsync(v + 2 * p.n, inc, sizeof(double2) * p.nfp, cudaMemcpyHostToDevice, c.stream));
            dinc = v + 2 * p.n;
        }
        evaluate_field(c, p, v, v + p.n, dinc, v + 2 * p.n + p.nfp);
        to_host(c, out, v + 2 * p.n + p.nfp, sizeof(double2) * p.nfp);
    });
}

BEM_API bem_status bem_convert_to_pressure(const bem_problem* pp, double frequency, bem_cplx* v, int64_t n) {
    if (!pp || (!v && n)) return BEM_ERR_BAD_INPUT;
    double omega = 2.0 * 3.14159265358979323846 * frequency;
    cd s = {0.0, omega * pp->p.in.mass_density};
    for (int64_t i = 0; i < n; ++i) {
        cd r = cmulh({v[i].re, v[i].im}, s);
        v[i].re = r.re;
        v[i].im = r.im;
    }
    return BEM_OK;
}

BEM_API bem_status bem_run_batch(bem_ctx* ctx, bem_problem* const* problems, int nprob, bem_precond precond,
                                 bem_cplx* const* scattered, bem_cplx* const* incident,
                                 bem_solve_report* const* reports, int check_vs_lu, int64_t max_operator_bytes) {
    if (!ctx || !problems || nprob < 0 || max_operator_bytes < 0) return BEM_ERR_BAD_INPUT;
    for (int i = 0; i < nprob; ++i)
        if (!problems[i]) return BEM_ERR_BAD_INPUT;
    return guard(ctx, [&] {
        Context& c = ctx->c;
        set_device(c);
        std::vector<Problem*> probs;
        for (int i = 0; i < nprob; ++i) {
            Problem& p = problems[i]->p;
            probs.push_back(&p);
            if (reports && reports[i])
                for (size_t f = 0; f < p.freqs.size(); ++f) {
                    std::memset(&reports[i][f], 0, sizeof(bem_solve_report));
                    reports[i][f].rel_err_vs_lu = -1;
                }
        }
        if (nprob == 0) return;
        run_mixed_batch(c, probs, precond, scattered, incident, reports, check_vs_lu != 0,
                        (size_t)max_operator_bytes);
    });
}

BEM_API bem_status bem_run(bem_ctx* ctx, bem_problem* pp, bem_form form, bem_precond precond, bem_cplx* scattered,
                           bem_cplx* incident, bem_solve_report* reports, int check_vs_lu) {
    if (!ctx || !pp) return BEM_ERR_BAD_INPUT;
    return guard(ctx, [&] {
        Context& c = ctx->c;
        Problem& p = pp->p;
        set_device(c);
        int64_t nf = (int64_t)p.freqs.size();
        if (reports)
            for (int64_t f = 0; f < nf * p.nrhs(); ++f) {
                std::memset(&reports[f], 0, sizeof(bem_solve_report));
                reports[f].rel_err_vs_lu = -1;
            }
        if (form == BEM_FORM_MIXED || form == BEM_FORM_REFINED || form == BEM_FORM_MIXED_ROUNDED) {
            run_mixed(c, p, precond, scattered, incident, reports, check_vs_lu != 0, form == BEM_FORM_REFINED,
                      form == BEM_FORM_MIXED_ROUNDED);
            return;
        }
        // analysis.rs:87-111, one frequency at a time
        int64_t n = p.n, nfp = p.nfp;
        DevBuf b;
        b.ensure(sizeof(double2) * (3 * n + 2 * nfp + 2));
        double2* rhs = b.as<double2>();
        double2* phi = rhs + n;
        double2* vn = phi + n;
        double2* inc = vn + n;
        double2* fps = inc + nfp;
        const int64_t nrhs = p.nrhs();
        c.last_phi.assign((size_t)(2 * n * nf * nrhs), 0.0);
        c.last_vn.assign((size_t)(2 * n * nf * nrhs), 0.0);
        c.last_n = n;
        c.last_nf = nf;
        int64_t saved = p.ifreq;
        // every right-hand side as the reference would run it; with the
        // Direct solver the waves of a frequency share its LU factorization
        // (the same factors and the same answer as factoring per wave)
        for (int64_t f0 = 0; f0 < nf; ++f0)
        for (int64_t r = 0; r < nrhs; ++r) {
            p.select_rhs(r);
            p.ifreq = f0;
            const int64_t f = r * nf + f0;  // output slot
            auto t0 = std::chrono::steady_clock::now();
            incident_surface(c, p, rhs);
            bem_solve_report* rep = reports ? &reports[f] : nullptr;
            if (p.in.solver == 2) solve_surface_hmatrix(c, p, rhs, phi, vn, rep);
            else solve_surface_dense_fp64(c, p, rhs, phi, vn, rep, nullptr, r > 0 && !check_vs_lu);
            incident_field(c, p, inc);
            evaluate_field(c, p, phi, vn, p.in.output_total ? inc : nullptr, fps);
            std::vector<double2> hs((size_t)nfp), hi((size_t)nfp);
            to_host(c, hs.data(), fps, sizeof(double2) * nfp);
            to_host(c, hi.data(), inc, sizeof(double2) * nfp);
            to_host(c, c.last_phi.data() + 2 * n * f, phi, sizeof(double2) * n);
            to_host(c, c.last_vn.data() + 2 * n * f, vn, sizeof(double2) * n);
            if (rep) rep->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            if (check_vs_lu && rep) rep->rel_err_vs_lu = lu_reference_error(c, p, c.last_phi.data() + 2 * n * f,
                                                                             c.last_vn.data() + 2 * n * f);
            // postprocess.rs:70-79
            double s = p.in.output_pressure ? p.omega() * p.in.mass_density : 0.0;
            for (int64_t i = 0; i < nfp; ++i) {
                double2 a = hs[(size_t)i], q = hi[(size_t)i];
                if (p.in.output_pressure) {
                    a = make_double2(-a.y * s, a.x * s);
                    q = make_double2(-q.y * s, q.x * s);
                }
                if (scattered) { scattered[f * nfp + i].re = a.x; scattered[f * nfp + i].im = a.y; }
                if (incident) { incident[f * nfp + i].re = q.x; incident[f * nfp + i].im = q.y; }
            }
        }
        p.select_rhs(0);
        p.ifreq = saved;
    });
}

BEM_API bem_status bem_learned_train(bem_ctx* ctx, bem_problem* const* problems, int nproblems, int steps,
                                     int nprobe, double lr, uint64_t seed, double* losses) {
    if (!ctx || !problems || nproblems < 1 || steps < 0 || nprobe < 1) return BEM_ERR_BAD_INPUT;
    return guard(ctx, [&] {
        set_device(ctx->c);
        std::vector<Problem*> ps;
        for (int i = 0; i < nproblems; ++i) {
            require(problems[i] != nullptr, "null problem");
            ps.push_back(&problems[i]->p);
        }
        std::vector<double> l;
        learned_train(ctx->c, ps, steps, nprobe, lr, seed, l);
        if (losses) std::memcpy(losses, l.data(), sizeof(double) * l.size());
    });
}

BEM_API int64_t bem_learned_num_params(void) { return learned_num_params(); }

BEM_API bem_status bem_learned_get_weights(bem_ctx* ctx, float* w) {
    if (!ctx || !w) return BEM_ERR_BAD_INPUT;
    return guard(ctx, [&] {
        require(ctx->c.net && ctx->c.net->ready, "no network loaded");
        set_device(ctx->c);
        BEM_CUDA(cudaMemcpyAsync(w, ctx->c.net->w.p, sizeof(float) * learned_num_params(), cudaMemcpyDeviceToHost,
                                 ctx->c.stream));
        ctx->c.sync();
    });
}

BEM_API bem_status bem_learned_set_weights(bem_ctx* ctx, const float* w) {
    if (!ctx || !w) return BEM_ERR_BAD_INPUT;
    return guard(ctx, [&] {
        set_device(ctx->c);
        if (!ctx->c.net) ctx->c.net = std::make_shared<LearnedNet>();
        LearnedNet& net = *ctx->c.net;
        if (!net.ready) net.init(ctx->c, 0);
        net.w_host.assign(w, w + learned_num_params());
        net.upload(ctx->c);
        BEM_CUDA(cudaMemsetAsync(net.m1.p, 0, sizeof(float) * learned_num_params(), ctx->c.stream));
        BEM_CUDA(cudaMemsetAsync(net.m2.p, 0, sizeof(float) * learned_num_params(), ctx->c.stream));
        net.step = 0;
        ctx->c.sync();
    });
}

BEM_API bem_status bem_learned_mlp_eval(bem_ctx* ctx, int64_t P, const float* features, const float* dO, float* out,
                                        float* grad) {
    if (!ctx || P < 1 || !features) return BEM_ERR_BAD_INPUT;
    return guard(ctx, [&] {
        set_device(ctx->c);
        learned_mlp_eval(ctx->c, P, features, dO, out, grad);
    });
}

BEM_API bem_status bem_learned_mlp_infer(bem_ctx* ctx, int64_t P, const float* features, float* out) {
    if (!ctx || P < 1 || !features || !out) return BEM_ERR_BAD_INPUT;
    return guard(ctx, [&] {
        set_device(ctx->c);
        learned_mlp_infer(ctx->c, P, features, out);
    });
}

BEM_API bem_status bem_last_surface(bem_ctx* ctx, const bem_problem* pp, bem_cplx* phi, bem_cplx* vn) {
    if (!ctx || !pp) return BEM_ERR_BAD_INPUT;
    Context& c = ctx->c;
    if (c.last_n != pp->p.n || c.last_phi.empty()) return BEM_ERR_BAD_INPUT;
    if (phi) std::memcpy(phi, c.last_phi.data(), sizeof(double) * c.last_phi.size());
    if (vn) std::memcpy(vn, c.last_vn.data(), sizeof(double) * c.last_vn.size());
    return BEM_OK;
}

}  // extern "C"
