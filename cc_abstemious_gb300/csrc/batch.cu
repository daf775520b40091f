// Several bodies in one batch (mixed form).  The reference runs one Analysis
// per body and one frequency at a time (analysis.rs:87-111); here every
// frequency of every body is assembled by one multi-body launch and all
// systems are solved by one ragged batched GMRES (systems of different sizes
// side by side, CUDA-graph captured), so small bodies do not leave the GPU
// idle.  Bodies are grouped into chunks whose operators fit a share of the
// free device memory.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <optional>

#include "common.cuh"
#include "complex.cuh"
#include "gmres.cuh"
#include "mixed.cuh"
#include "precond.cuh"

namespace bem {

namespace {

struct BodyPlan {
    Problem* p;
    int index;  // position in the caller's arrays
    int nf;
    int64_t n, ld, nfp;
    std::vector<double> ks;
    std::vector<cd> al, be, ga, de;
    bool need_rowsum;
    int m;
    int64_t max_restarts;
    double tol;
    size_t op_bytes;
};

void plan_body(Problem& p, BodyPlan& b) {
    b.p = &p;
    b.nf = (int)p.freqs.size();
    b.n = p.n;
    b.ld = p.geo.npad;
    b.nfp = p.nfp;
    const int64_t saved = p.ifreq;
    b.ks.resize((size_t)b.nf);
    b.al.resize((size_t)b.nf);
    b.be.resize((size_t)b.nf);
    b.ga.resize((size_t)b.nf);
    b.de.resize((size_t)b.nf);
    for (int f = 0; f < b.nf; ++f) {
        p.ifreq = f;
        b.ks[(size_t)f] = p.wavenumber();
        lhs_factors(p, b.al[(size_t)f], b.be[(size_t)f]);
        rhs_factors(p, b.ga[(size_t)f], b.de[(size_t)f]);
    }
    p.ifreq = saved;
    b.need_rowsum = !(p.in.bc_value[0] == 0.0 && p.in.bc_value[1] == 0.0) && p.in.bc_type != 2;
    // the problem's GMRES settings, or for the direct solver a tight
    // tolerance (the mixed form always iterates), as in the one-body form
    int64_t max_it = p.in.solver == 0 ? 1000 : p.in.max_iterations;
    double tol = p.in.solver == 0 ? 1e-10 : p.in.tolerance;
    if (max_it <= 0) max_it = 1000;
    if (max_it > b.n) max_it = b.n;
    if (tol <= 0) tol = 1e-5;
    b.m = (int)std::ceil(std::sqrt((double)max_it));
    b.max_restarts = max_it / b.m;
    b.tol = tol;
    b.op_bytes = sizeof(float2) * (size_t)b.ld * (size_t)b.n * (size_t)b.nf;
}

namespace {
// Wall time of one part of a batch solve (synchronised at its end) for the
// library's per-stage profile.
struct BatchStage {
    Context& c;
    const char* name;
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    int64_t l0;
    BatchStage(Context& ctx, const char* n) : c(ctx), name(n), l0(ctx.launches) {}
    ~BatchStage() {
        if (!c.profiling) return;
        cudaStreamSynchronize(c.stream);
        c.stage_add(name, std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count(),
                    c.launches - l0, 0);
    }
};
}  // namespace

void solve_chunk(Context& c, std::vector<BodyPlan*>& bodies, bem_precond precond, bem_cplx* const* scattered,
                 bem_cplx* const* incident, bem_solve_report* const* reports, bool check_vs_lu) {
    auto t_start = std::chrono::steady_clock::now();
    // systems body-major, frequency-minor
    std::vector<int64_t> ns, lds;
    std::vector<size_t> aoff;
    std::vector<int> sys_body, ms;
    std::vector<double> tols, ks;
    std::vector<int64_t> maxr;
    std::vector<size_t> body_sys0;
    size_t ent = 0;
    int mmax = 1;
    for (size_t b = 0; b < bodies.size(); ++b) {
        BodyPlan& B = *bodies[b];
        body_sys0.push_back(ns.size());
        for (int f = 0; f < B.nf; ++f) {
            ns.push_back(B.n);
            lds.push_back(B.ld);
            aoff.push_back(ent);
            ent += (size_t)B.ld * (size_t)B.n;  // ld is a multiple of 64: aligned float4 columns
            sys_body.push_back((int)b);
            ms.push_back(B.m);
            tols.push_back(B.tol);
            ks.push_back(B.ks[(size_t)f]);
            maxr.push_back(B.max_restarts);
        }
        mmax = std::max(mmax, B.m);
    }
    const size_t nsys = ns.size();
    c.w_mat.ensure(sizeof(float2) * ent);
    float2* A = c.w_mat.as<float2>();
    GmWorkspace ws;
    ws.mem_pool = &c.w_gm;
    ws.z_pool = &c.w_gmz;
    gm_prepare_ragged(c, ws, ns, lds, aoff, mmax, A, true);
    const std::vector<GmSys>& L = ws.sys_host;
    const size_t vtot = L.back().v_off + (size_t)L.back().n;
    size_t fptot = 0;
    std::vector<size_t> fpoff(nsys);
    for (size_t s = 0; s < nsys; ++s) {
        fpoff[s] = fptot;
        fptot += (size_t)bodies[(size_t)sys_body[s]]->nfp;
    }
    c.w_vec.ensure(sizeof(double2) * (4 * vtot + 2 * fptot + 2));
    double2* inc = c.w_vec.as<double2>();
    double2* rowsum = inc + vtot;
    double2* phi = rowsum + vtot;
    double2* vn = phi + vtot;
    double2* finc = vn + vtot;
    double2* fps = finc + fptot;

    // ---- assembly: one launch for every body without a boundary-value term;
    // bodies that need rowsum(gamma H + delta G) use the one-body kernel
    {
        BatchStage bs(c, "batch_assembly");
        std::vector<BodyAsm32> multi;
        std::vector<size_t> multi_sys0;
        for (size_t b = 0; b < bodies.size(); ++b) {
            BodyPlan& B = *bodies[b];
            const size_t s0 = body_sys0[b];
            if (B.need_rowsum) {
                assemble_system_fp32_body(c, *B.p, B.ks.data(), B.al.data(), B.be.data(), B.ga.data(), B.de.data(),
                                          B.nf, A + aoff[s0], B.ld, (size_t)B.ld * B.n, rowsum + L[s0].v_off,
                                          (size_t)B.n, ws.anorm + s0);
            } else {
                multi.push_back(BodyAsm32{B.p, B.nf, B.ks.data(), B.al.data(), B.be.data(), A + aoff[s0], B.ld,
                                          (size_t)B.ld * B.n});
                multi_sys0.push_back(s0);
            }
        }
        if (!multi.empty()) {
            // norms come out in the order of `multi`; scatter them when some
            // bodies were assembled separately
            const bool contiguous = multi.size() == bodies.size();
            DevBuf tmp;
            double* dst = ws.anorm;
            if (!contiguous) {
                tmp.ensure(sizeof(double) * nsys);
                dst = tmp.as<double>();
            }
            assemble_fp32_multi(c, multi, dst);
            if (!contiguous) {
                size_t g = 0;
                for (size_t i = 0; i < multi.size(); ++i) {
                    BEM_CUDA(cudaMemcpyAsync(ws.anorm + multi_sys0[i], dst + g, sizeof(double) * multi[i].nsys,
                                             cudaMemcpyDeviceToDevice, c.stream));
                    g += (size_t)multi[i].nsys;
                }
                c.sync();
            }
        }
    }
    // ---- right-hand sides
    std::optional<BatchStage> part;
    part.emplace(c, "batch_rhs");
    {
        std::vector<IncItem> items;
        for (size_t s = 0; s < nsys; ++s) {
            BodyPlan& B = *bodies[(size_t)sys_body[s]];
            const Problem& p = *B.p;
            items.push_back(IncItem{&p, (int64_t)(s - body_sys0[(size_t)sys_body[s]]), 0, false,
                                    inc + L[s].v_off, ws.bt.B + L[s].v_off, p.in.bc_type == 0 ? 1.0 : -1.0,
                                    {p.in.bc_value[0], p.in.bc_value[1]},
                                    B.need_rowsum ? rowsum + L[s].v_off : nullptr});
        }
        incident_batch(c, items);
    }
    part.reset();
    // ---- batched GMRES over every system
    gm_init_each(c, ws, tols, maxr, ms);
    if (precond != BEM_PRECOND_NONE) {
        std::vector<Problem*> probs;
        for (BodyPlan* B : bodies) probs.push_back(B->p);
        precond = precond_setup_multi(c, probs, sys_body, ws, precond, ks.data());
    }
    int64_t cap = 0;
    for (size_t s = 0; s < nsys; ++s) cap = std::max(cap, maxr[s] * (int64_t)ms[s] + 1);
    std::vector<GmState> st;
    {
        BatchStage bs(c, "batch_gmres");
        gm_run(c, ws, c.profiling ? 0 : 4, cap);
        gm_read_states(c, ws, st);
    }
    // ---- surface unknowns and field points
    part.emplace(c, "batch_field");
    {
        std::vector<UnpackItem> un;
        std::vector<IncItem> fi;
        for (size_t s = 0; s < nsys; ++s) {
            BodyPlan& B = *bodies[(size_t)sys_body[s]];
            const int64_t f = (int64_t)(s - body_sys0[(size_t)sys_body[s]]);
            un.push_back(UnpackItem{B.p, f, ws.bt.X + L[s].v_off, phi + L[s].v_off, vn + L[s].v_off});
            if (B.nfp) fi.push_back(IncItem{B.p, f, 0, true, finc + fpoff[s], nullptr, 0.0, {0, 0}, nullptr});
        }
        unpack_batch(c, un);
        incident_batch(c, fi);
    }
    for (size_t b = 0; b < bodies.size(); ++b) {
        BodyPlan& B = *bodies[b];
        const size_t s0 = body_sys0[b];
        if (B.nfp)
            evaluate_field32_batch(c, *B.p, B.ks.data(), B.nf, phi + L[s0].v_off, vn + L[s0].v_off, B.n,
                                   B.p->in.output_total ? finc + fpoff[s0] : nullptr, fps + fpoff[s0]);
    }
    std::vector<double2> hs(fptot), hi(fptot), hphi(vtot), hvn(vtot);
    if (fptot) {
        BEM_CUDA(cudaMemcpyAsync(hs.data(), fps, sizeof(double2) * fptot, cudaMemcpyDeviceToHost, c.stream));
        BEM_CUDA(cudaMemcpyAsync(hi.data(), finc, sizeof(double2) * fptot, cudaMemcpyDeviceToHost, c.stream));
    }
    if (check_vs_lu) {
        BEM_CUDA(cudaMemcpyAsync(hphi.data(), phi, sizeof(double2) * vtot, cudaMemcpyDeviceToHost, c.stream));
        BEM_CUDA(cudaMemcpyAsync(hvn.data(), vn, sizeof(double2) * vtot, cudaMemcpyDeviceToHost, c.stream));
    }
    c.sync();
    part.reset();
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
    for (size_t s = 0; s < nsys; ++s) {
        const int bi = sys_body[s];
        BodyPlan& B = *bodies[(size_t)bi];
        Problem& p = *B.p;
        const int f = (int)(s - body_sys0[(size_t)bi]);
        p.ifreq = f;
        const double w = p.in.output_pressure ? p.omega() * p.in.mass_density : 0.0;
        bem_cplx* so = scattered ? scattered[B.index] : nullptr;
        bem_cplx* io = incident ? incident[B.index] : nullptr;
        for (int64_t i = 0; i < B.nfp; ++i) {
            double2 a = hs[fpoff[s] + (size_t)i], q = hi[fpoff[s] + (size_t)i];
            if (p.in.output_pressure) {
                a = make_double2(-a.y * w, a.x * w);
                q = make_double2(-q.y * w, q.x * w);
            }
            if (so) { so[f * B.nfp + i].re = a.x; so[f * B.nfp + i].im = a.y; }
            if (io) { io[f * B.nfp + i].re = q.x; io[f * B.nfp + i].im = q.y; }
        }
        if (reports && reports[B.index]) {
            bem_solve_report& r = reports[B.index][f];
            r.num_mv = st[s].num_mv;
            r.restarts = st[s].restarts + (st[s].converged ? 1 : 0);
            r.iterations = st[s].iterations;
            r.backward_error = st[s].error;
            r.flag = st[s].converged ? 1 : 2;
            r.precond = (int32_t)precond;
            r.seconds = secs / (double)nsys;
            r.rel_err_vs_lu = -1;
            if (check_vs_lu)
                r.rel_err_vs_lu = lu_reference_error(c, p, reinterpret_cast<const double*>(hphi.data() + L[s].v_off),
                                                     reinterpret_cast<const double*>(hvn.data() + L[s].v_off));
        }
    }
    for (BodyPlan* B : bodies) B->p->ifreq = 0;
}

}  // namespace

void run_mixed_batch(Context& c, const std::vector<Problem*>& probs, bem_precond precond,
                     bem_cplx* const* scattered, bem_cplx* const* incident, bem_solve_report* const* reports,
                     bool check_vs_lu, size_t budget_bytes) {
    c.stages.clear();
    std::vector<BodyPlan> plans(probs.size());
    std::vector<BodyPlan*> batched;
    for (size_t i = 0; i < probs.size(); ++i) {
        Problem& p = *probs[i];
        require(!p.freqs.empty(), "no frequencies");
        // a first-kind operator (classical formulation, pressure condition)
        // keeps an FP64 operator: solved body by body as in bem_run
        if (p.in.method_type == 0 && p.in.bc_type == 0) {
            run_mixed(c, p, precond, scattered ? scattered[i] : nullptr, incident ? incident[i] : nullptr,
                      reports ? reports[i] : nullptr, check_vs_lu);
            continue;
        }
        plan_body(p, plans[i]);
        plans[i].index = (int)i;
        batched.push_back(&plans[i]);
    }
    if (batched.empty()) return;
    if (budget_bytes == 0) {
        size_t fr = 0, tot = 0;
        BEM_CUDA(cudaMemGetInfo(&fr, &tot));
        // operators take most of a chunk's memory; GMRES bases, the
        // preconditioner blocks and the vectors share the rest
        budget_bytes = (size_t)(0.6 * (double)(fr + c.w_mat.bytes));
    }
    // largest bodies first: chunks of similar sizes, and the large systems
    // start their tiles early in every mat-vec launch
    std::stable_sort(batched.begin(), batched.end(),
                     [](const BodyPlan* a, const BodyPlan* b) { return a->n > b->n; });
    size_t i = 0;
    while (i < batched.size()) {
        std::vector<BodyPlan*> chunk;
        size_t bytes = 0;
        // the LU preconditioner keeps a factored copy of every operator and,
        // per unknown, the diagonal blocks and the panel workspaces (19 KB, or
        // 38 KB where eight-step groups are allowed)
        auto need = [&](const BodyPlan* p) {
            return precond == BEM_PRECOND_LU
                       ? 2.0 * (double)p->op_bytes + lu_bytes_per_unknown(p->n) * (double)p->n * (double)p->nf
                       : (double)p->op_bytes;
        };
        while (i < batched.size() && (chunk.empty() || (double)bytes + need(batched[i]) <= (double)budget_bytes)) {
            bytes += (size_t)need(batched[i]);
            chunk.push_back(batched[i]);
            ++i;
        }
        solve_chunk(c, chunk, precond, scattered, incident, reports, check_vs_lu);
    }
}

}  // namespace bem
