// Mixed-precision batched form: every frequency of a body is assembled in one
// single-precision pass (float-float geometry and phase, FP64 singular self
// term), then all systems are solved together by the batched FP64 restarted
// GMRES over the FP32 operators (compensated mat-vecs), and the field points
// are evaluated in FP64.  The error against an FP64 LU of the same operator is
// measured on request, outside any timed region.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>

#include "common.cuh"
#include "complex.cuh"
#include "gmres.cuh"
#include "hmixed.cuh"
#include "hmatrix.cuh"
#include "mixed.cuh"
#include "precond.cuh"

namespace bem {

namespace {
struct EventTimer {
    cudaEvent_t a = nullptr, b = nullptr;
    Context& c;
    bool on;
    explicit EventTimer(Context& ctx) : c(ctx), on(ctx.profiling) {
        if (on) {
            BEM_CUDA(cudaEventCreate(&a));
            BEM_CUDA(cudaEventCreate(&b));
            BEM_CUDA(cudaEventRecord(a, c.stream));
        }
    }
    void stop(const std::string& name, int64_t launches, double bytes) {
        if (!on) return;
        BEM_CUDA(cudaEventRecord(b, c.stream));
        BEM_CUDA(cudaEventSynchronize(b));
        float ms = 0;
        BEM_CUDA(cudaEventElapsedTime(&ms, a, b));
        c.stage_add(name, ms, launches, bytes);
    }
    ~EventTimer() {
        if (a) cudaEventDestroy(a);
        if (b) cudaEventDestroy(b);
    }
};
}  // namespace

double lu_reference_error(Context& c, const Problem& p, const double* phi_host, const double* vn_host) {
    int64_t n = p.n;
    DevBuf b, A;
    b.ensure(sizeof(double2) * 3 * n);
    A.ensure(sizeof(double2) * (size_t)n * n);
    double2* inc = b.as<double2>();
    double2* phi = inc + n;
    double2* vn = phi + n;
    incident_surface(c, p, inc);
    Problem q;  // same operator, solved with the direct FP64 LU
    Problem& pp = const_cast<Problem&>(p);
    int saved = pp.in.solver;
    pp.in.solver = 0;
    try {
        solve_surface_dense_fp64(c, pp, inc, phi, vn, nullptr, A.as<double2>());
    } catch (...) {
        pp.in.solver = saved;
        throw;
    }
    pp.in.solver = saved;
    std::vector<double> ref(2 * n);
    const double* mine = p.in.bc_type == 0 ? vn_host : phi_host;
    BEM_CUDA(cudaMemcpyAsync(ref.data(), p.in.bc_type == 0 ? (void*)vn : (void*)phi, sizeof(double2) * n,
                             cudaMemcpyDeviceToHost, c.stream));
    c.sync();
    double num = 0, den = 0;
    for (int64_t i = 0; i < 2 * n; ++i) {
        double d = mine[i] - ref[i];
        num += d * d;
        den += ref[i] * ref[i];
    }
    (void)q;
    return std::sqrt(num / den);
}

// out[s] = in[s / R]: the norm of each frequency's operator for its R systems.
__global__ void repeat_norms_kernel(const double* __restrict__ in, int R, int ns, double* __restrict__ out) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < ns) out[s] = in[s / R];
}

// Frequencies [F0, F0 + nf) of the problem as one batch.  With several
// right-hand sides (R incident waves) every frequency's operator is assembled
// once and shared by its R systems (s = f R + r) through the ragged batch
// layout; the LU preconditioner factors it once.
static void run_mixed_range(Context& c, Problem& p, int64_t F0, int64_t nf, bem_precond precond,
                            bem_cplx* scattered, bem_cplx* incident, bem_solve_report* reports, bool check_vs_lu,
                            bool fp64_operator, bool rounded) {
    const int64_t n = p.n, nfp = p.nfp, R = p.nrhs(), ns = nf * R, NF = (int64_t)p.freqs.size();
    const int64_t ld = p.geo.npad;  // multiple of 64: aligned float4 loads
    const size_t mstride = (size_t)ld * n;
    const int64_t saved_ifreq = p.ifreq;
    auto t_start = std::chrono::steady_clock::now();

    // per-frequency factors (influence_matrix.rs:130-162)
    std::vector<double> ks(nf), ks_sys(ns);
    std::vector<cd> al(nf), be(nf), ga(nf), de(nf);
    for (int64_t f = 0; f < nf; ++f) {
        p.ifreq = F0 + f;
        ks[f] = p.wavenumber();
        lhs_factors(p, al[f], be[f]);
        rhs_factors(p, ga[f], de[f]);
        for (int64_t r = 0; r < R; ++r) ks_sys[f * R + r] = ks[f];
    }
    const bool need_rowsum = !(p.in.bc_value[0] == 0.0 && p.in.bc_value[1] == 0.0) && p.in.bc_type != 2;

    // A first-kind operator (classical formulation with a pressure condition:
    // the single layer G alone) is too ill-conditioned for single-precision
    // storage at 1e-6; those systems keep an FP64 operator in the same batch,
    // as every operator of the refined form does.
    const bool first_kind = fp64_operator || (p.in.method_type == 0 && p.in.bc_type == 0);
    // the Hierarchical solver: ACA-compressed operators with FP32 factors
    // instead of dense ones (hmixed.cu)
    const bool hier = p.in.solver == 2 && !first_kind;
    // FP64 operators assembled in one pass are kept split: their FP32
    // rounding and the FP32 rounding of the remainder, the same 16 bytes per
    // entry, applied in float-float on the FP32 pipe (gmres.cu)
    const bool split = first_kind && !need_rowsum;
    if (!hier) c.w_mat.ensure((first_kind ? sizeof(double2) : sizeof(float2)) * mstride * nf);
    float2* A32 = c.w_mat.as<float2>();
    double2* A64 = c.w_mat.as<double2>();
    c.w_vec.ensure(sizeof(double2) * ((size_t)ns * (3 * n + 2 * nfp) + (size_t)nf * n + 2) + sizeof(double) * nf);
    double2* inc = c.w_vec.as<double2>();
    double2* rowsum = inc + ns * n;
    double2* phi = rowsum + nf * n;
    double2* vn = phi + ns * n;
    double2* finc = vn + ns * n;
    double2* fps = finc + ns * nfp;
    double* normf = reinterpret_cast<double*>(fps + ns * nfp + 2);

    // solver parameters: the problem's GMRES settings, or for the direct
    // solver a tight tolerance (the mixed form always iterates)
    int64_t max_it = p.in.solver == 0 ? 1000 : p.in.max_iterations;
    double tol = p.in.solver == 0 ? 1e-10 : p.in.tolerance;
    if (max_it <= 0) max_it = 1000;
    if (max_it > n) max_it = n;
    if (tol <= 0) tol = 1e-5;
    int m = (int)std::ceil(std::sqrt((double)max_it));
    int64_t restarts = max_it / m;
    GmWorkspace ws;
    ws.mem_pool = &c.w_gm;
    ws.z_pool = &c.w_gmz;
    const void* Aop = first_kind ? (const void*)A64 : (const void*)A32;
    std::shared_ptr<HMixed> Hm;
    if (hier) {
        gm_prepare(c, ws, (int)ns, n, m, nullptr, n, 0, true, false);
    } else if (R == 1) {
        gm_prepare(c, ws, (int)nf, n, m, Aop, ld, split ? 2 * mstride : mstride, !first_kind || split, false);
    } else {
        std::vector<int64_t> nsz((size_t)ns, n), lds((size_t)ns, ld);
        std::vector<size_t> aoff((size_t)ns);
        for (int64_t s = 0; s < ns; ++s) aoff[(size_t)s] = (size_t)(s / R) * (split ? 2 * mstride : mstride);
        gm_prepare_ragged(c, ws, nsz, lds, aoff, m, Aop, !first_kind || split);
    }
    if (split) {
        ws.bt.split_lo = (int64_t)mstride;
        ws.mv_stage = "gmres_matvec_split";
        ws.mv_bytes = 16.0 * (double)n * (double)n;
    }

    if (hier) {
        EventTimer t(c);
        Hm = hmixed_build(c, p, F0, nf, (int)R);
        hmixed_attach(c, ws, Hm);
        const HMixedStats hs = hmixed_stats(*Hm);
        ws.mv_bytes = 8.0 * (double)hs.store_entries / (double)nf;  // per system and mat-vec
        ws.mv_stage = "gmres_matvec_hmatrix";
        if (need_rowsum)
            for (int64_t f = 0; f < nf; ++f) {
                p.ifreq = F0 + f;
                hmatrix_row_sums(c, p, 0, rowsum + f * n);
            }
        t.stop("hmatrix_build", nf, 8.0 * (double)hs.store_entries);
    } else if (split) {
        // every frequency in one pass, in float-float, norms accumulated by
        // the kernel
        EventTimer t(c);
        assemble_system_split(c, p, ks.data(), al.data(), be.data(), (int)nf, reinterpret_cast<float2*>(A64), ld,
                              mstride, R == 1 ? ws.anorm : normf);
        if (R > 1) {
            repeat_norms_kernel<<<(unsigned)((ns + 127) / 128), 128, 0, c.stream>>>(normf, (int)R, (int)ns, ws.anorm);
            BEM_CHECK_LAUNCH(&c);
        }
        t.stop("assemble_split", (nf + 15) / 16, 16.0 * (double)n * n * nf);
    } else if (first_kind) {
        EventTimer t(c);
        for (int64_t f = 0; f < nf; ++f) {
            p.ifreq = F0 + f;
            assemble_system_fp64(c, p, A64 + f * mstride, ld, al[f], be[f], ga[f], de[f],
                                 need_rowsum ? rowsum + f * n : nullptr);
        }
        gm_matrix_norms(c, ws);
        t.stop("assemble_fp64", nf, 16.0 * (double)n * n * nf);
    } else if (rounded && !need_rowsum) {
        // the FP32 operator rounded once from its float-float value (the
        // refined form's assembly without the remainder plane)
        EventTimer t(c);
        assemble_system_split(c, p, ks.data(), al.data(), be.data(), (int)nf, A32, ld, mstride,
                              R == 1 ? ws.anorm : normf, false);
        if (R > 1) {
            repeat_norms_kernel<<<(unsigned)((ns + 127) / 128), 128, 0, c.stream>>>(normf, (int)R, (int)ns, ws.anorm);
            BEM_CHECK_LAUNCH(&c);
        }
        t.stop("assemble_rounded", (nf + 15) / 16, 8.0 * (double)n * n * nf);
    } else {
        // the assembly kernel also writes ||A_f||_F for the stopping test
        EventTimer t(c);
        assemble_system_fp32_body(c, p, ks.data(), al.data(), be.data(), ga.data(), de.data(), (int)nf, A32, ld,
                                  mstride, need_rowsum ? rowsum : nullptr, (size_t)n, R == 1 ? ws.anorm : normf);
        if (R > 1) {
            repeat_norms_kernel<<<(unsigned)((ns + 127) / 128), 128, 0, c.stream>>>(normf, (int)R, (int)ns, ws.anorm);
            BEM_CHECK_LAUNCH(&c);
        }
        t.stop("assemble_fp32", (nf + 15) / 16, 8.0 * (double)n * n * nf);
    }
    {
        EventTimer t(c);
        for (int64_t s = 0; s < ns; ++s) {
            p.select_rhs(s % R);
            p.ifreq = F0 + s / R;
            incident_surface(c, p, inc + s * n);
        }
        t.stop("incident", ns, 0);
    }

    const double sgn = p.in.bc_type == 0 ? 1.0 : -1.0;
    for (int64_t s = 0; s < ns; ++s)
        launch_rhs_combine(c, n, sgn, inc + s * n, {p.in.bc_value[0], p.in.bc_value[1]},
                           need_rowsum ? rowsum + (s / R) * n : nullptr, ws.bt.B + s * n);
    std::vector<GmState> st;
    {
        EventTimer t(c);
        gm_init(c, ws, tol, restarts);
        if (precond != BEM_PRECOND_NONE && hier)
            // the compressed operators have no dense copy to factor: every
            // preconditioner request becomes block-Jacobi on the diagonal leaves
            precond = hmixed_block_jacobi(c, ws, Hm) ? BEM_PRECOND_BLOCK_JACOBI : BEM_PRECOND_NONE;
        else if (precond != BEM_PRECOND_NONE)
            precond = precond_setup(c, p, ws, precond, ks_sys.data());
        gm_run(c, ws, c.profiling ? 0 : 4, restarts * (int64_t)m + 1);
        gm_read_states(c, ws, st);
        int64_t mv = 0;
        for (auto& x : st) mv += x.num_mv;
        t.stop("gmres", mv, hier ? ws.mv_bytes * mv : (first_kind ? 16.0 : 8.0) * (double)n * n * mv);
    }
    {
        EventTimer t(c);
        for (int64_t s = 0; s < ns; ++s) {
            p.select_rhs(s % R);
            p.ifreq = F0 + s / R;
            unpack_solution(c, p, ws.bt.X + s * n, phi + s * n, vn + s * n);
            incident_field(c, p, finc + s * nfp);
        }
        evaluate_field32_batch(c, p, ks_sys.data(), (int)ns, phi, vn, n, p.in.output_total ? finc : nullptr, fps);
        t.stop("field", 1, 0);
    }
    std::vector<double2> hs((size_t)(ns * nfp)), hi((size_t)(ns * nfp));
    if (nfp) {
        BEM_CUDA(cudaMemcpyAsync(hs.data(), fps, sizeof(double2) * ns * nfp, cudaMemcpyDeviceToHost, c.stream));
        BEM_CUDA(cudaMemcpyAsync(hi.data(), finc, sizeof(double2) * ns * nfp, cudaMemcpyDeviceToHost, c.stream));
    }
    // output slot of system s: wave-major, then frequency
    auto slot = [&](int64_t s) { return (s % R) * NF + F0 + s / R; };
    for (int64_t s = 0; s < ns; ++s) {
        BEM_CUDA(cudaMemcpyAsync(c.last_phi.data() + 2 * n * slot(s), phi + s * n, sizeof(double2) * n,
                                 cudaMemcpyDeviceToHost, c.stream));
        BEM_CUDA(cudaMemcpyAsync(c.last_vn.data() + 2 * n * slot(s), vn + s * n, sizeof(double2) * n,
                                 cudaMemcpyDeviceToHost, c.stream));
    }
    c.sync();
    double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
    for (int64_t s = 0; s < ns; ++s) {
        p.ifreq = F0 + s / R;
        double w = p.in.output_pressure ? p.omega() * p.in.mass_density : 0.0;
        for (int64_t i = 0; i < nfp; ++i) {
            double2 a = hs[(size_t)(s * nfp + i)], q = hi[(size_t)(s * nfp + i)];
            if (p.in.output_pressure) {
                a = make_double2(-a.y * w, a.x * w);
                q = make_double2(-q.y * w, q.x * w);
            }
            const int64_t o = slot(s) * nfp + i;
            if (scattered) { scattered[o].re = a.x; scattered[o].im = a.y; }
            if (incident) { incident[o].re = q.x; incident[o].im = q.y; }
        }
        if (reports) {
            bem_solve_report& r = reports[slot(s)];
            r.num_mv = st[(size_t)s].num_mv;
            r.restarts = st[(size_t)s].restarts + (st[(size_t)s].converged ? 1 : 0);
            r.iterations = st[(size_t)s].iterations;
            r.backward_error = st[(size_t)s].error;
            r.flag = st[(size_t)s].converged ? 1 : 2;
            r.precond = (int32_t)precond;
            r.seconds = secs / (double)ns;
            r.rel_err_vs_lu = -1;
        }
    }
    if (check_vs_lu && reports) {
        for (int64_t s = 0; s < ns; ++s) {
            p.select_rhs(s % R);
            p.ifreq = F0 + s / R;
            reports[slot(s)].rel_err_vs_lu = lu_reference_error(c, p, c.last_phi.data() + 2 * n * slot(s),
                                                                c.last_vn.data() + 2 * n * slot(s));
        }
    }
    p.select_rhs(0);
    p.ifreq = saved_ifreq;
}

void run_mixed(Context& c, Problem& p, bem_precond precond, bem_cplx* scattered, bem_cplx* incident,
               bem_solve_report* reports, bool check_vs_lu, bool fp64_operator, bool rounded) {
    c.stages.clear();
    const int64_t nf = (int64_t)p.freqs.size(), n = p.n;
    require(nf >= 1, "no frequencies");
    c.last_phi.assign((size_t)(2 * n * nf * p.nrhs()), 0.0);
    c.last_vn.assign((size_t)(2 * n * nf * p.nrhs()), 0.0);
    c.last_n = n;
    c.last_nf = nf;
    // frequencies per batch: the operators (and the LU copy) within 60% of the
    // device memory the context can use
    const bool op64 = fp64_operator || (p.in.method_type == 0 && p.in.bc_type == 0);
    const double ent = (double)p.geo.npad * (double)n;
    const double per = ent * (op64 ? 16.0 : 8.0) + (precond == BEM_PRECOND_LU ? ent * 8.0 + lu_bytes_per_unknown(n) * n : 0.0);
    size_t fr = 0, tot = 0;
    BEM_CUDA(cudaMemGetInfo(&fr, &tot));
    const double budget = 0.6 * (double)(fr + c.w_mat.bytes + c.w_lu_F.bytes);
    // (compressed operators: every frequency at once)
    const bool hier = p.in.solver == 2 && !op64;
    const int64_t chunk = hier ? nf : std::max<int64_t>(1, std::min<int64_t>(nf, (int64_t)(budget / per)));
    for (int64_t f0 = 0; f0 < nf; f0 += chunk)
        run_mixed_range(c, p, f0, std::min(chunk, nf - f0), precond, scattered, incident, reports, check_vs_lu,
                        fp64_operator, rounded);
}

}  // namespace bem
