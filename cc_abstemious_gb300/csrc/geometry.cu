// Collocation geometry (elements.rs:42-181 + preprocess.rs:126-153) and the
// incident wave (incident_wave.rs:7-99) on the device.
#include "common.cuh"
#include "complex.cuh"

namespace bem {

// One thread per collocation point.  Arithmetic uses explicitly rounded
// operations (no fused multiply-add) so the geometry is bit-identical to a
// sequential FP64 evaluation of the reference formulas.
__global__ void collocation_kernel(int64_t n, const double* __restrict__ nodes,
                                   const int32_t* __restrict__ etype, const int64_t* __restrict__ enodes,
                                   int64_t npad, double* __restrict__ geo) {
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= npad) return;
    double* x = geo;
    if (t >= n) {  // zero padding
        for (int k = 0; k < GEO_NARR; ++k) geo[k * npad + t] = 0.0;
        return;
    }
    const int64_t* nd = enodes + 4 * t;
    double c[3] = {0, 0, 0}, nrm[3], area, wt;
    if (etype[t] == 5) {
        // TRIGP1: xi = eta = 1/3, N = (1 - xi - eta, xi, eta), w = 1
        const double third = 1.0 / 3.0;
        double sf[3] = {__dsub_rn(__dsub_rn(1.0, third), third), third, third};
        for (int a = 0; a < 3; ++a)
            for (int k = 0; k < 3; ++k) c[k] = __dadd_rn(c[k], __dmul_rn(sf[a], nodes[3 * nd[a] + k]));
        const double* e0 = nodes + 3 * nd[0];
        const double* e1 = nodes + 3 * nd[1];
        const double* e2 = nodes + 3 * nd[2];
        double a_[3], b_[3];
        for (int k = 0; k < 3; ++k) { a_[k] = __dsub_rn(e1[k], e0[k]); b_[k] = __dsub_rn(e2[k], e0[k]); }
        nrm[0] = __dsub_rn(__dmul_rn(a_[1], b_[2]), __dmul_rn(a_[2], b_[1]));
        nrm[1] = __dsub_rn(__dmul_rn(a_[2], b_[0]), __dmul_rn(a_[0], b_[2]));
        nrm[2] = __dsub_rn(__dmul_rn(a_[0], b_[1]), __dmul_rn(a_[1], b_[0]));
        double nn = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(nrm[0], nrm[0]), __dmul_rn(nrm[1], nrm[1])),
                                         __dmul_rn(nrm[2], nrm[2])));
        area = __dmul_rn(0.5, nn);
        wt = 1.0;
    } else {
        // QUADGP1: xi = eta = 0, N = 1/4, dN carries 0.25, detJ another 0.25, w = 4
        const double dn[4][2] = {{-0.25, -0.25}, {0.25, -0.25}, {0.25, 0.25}, {-0.25, 0.25}};
        double dxi[3] = {0, 0, 0}, deta[3] = {0, 0, 0};
        for (int a = 0; a < 4; ++a)
            for (int k = 0; k < 3; ++k) {
                double X = nodes[3 * nd[a] + k];
                c[k] = __dadd_rn(c[k], __dmul_rn(0.25, X));
                dxi[k] = __dadd_rn(dxi[k], __dmul_rn(dn[a][0], X));
                deta[k] = __dadd_rn(deta[k], __dmul_rn(dn[a][1], X));
            }
        nrm[0] = __dsub_rn(__dmul_rn(dxi[1], deta[2]), __dmul_rn(dxi[2], deta[1]));
        nrm[1] = __dsub_rn(__dmul_rn(dxi[2], deta[0]), __dmul_rn(dxi[0], deta[2]));
        nrm[2] = __dsub_rn(__dmul_rn(dxi[0], deta[1]), __dmul_rn(dxi[1], deta[0]));
        double nn = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(nrm[0], nrm[0]), __dmul_rn(nrm[1], nrm[1])),
                                         __dmul_rn(nrm[2], nrm[2])));
        area = __dmul_rn(0.25, nn);
        wt = 4.0;
    }
    double nn = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(nrm[0], nrm[0]), __dmul_rn(nrm[1], nrm[1])),
                                     __dmul_rn(nrm[2], nrm[2])));
    x[GX * npad + t] = c[0];
    x[GY * npad + t] = c[1];
    x[GZ * npad + t] = c[2];
    x[GNX * npad + t] = __ddiv_rn(nrm[0], nn);
    x[GNY * npad + t] = __ddiv_rn(nrm[1], nn);
    x[GNZ * npad + t] = __ddiv_rn(nrm[2], nn);
    x[GAREA * npad + t] = area;
    x[GWT * npad + t] = wt;
    x[GWA * npad + t] = __dmul_rn(wt, area);
    double un[3] = {x[GNX * npad + t], x[GNY * npad + t], x[GNZ * npad + t]};
    double m = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(un[0], un[0]), __dmul_rn(un[1], un[1])),
                                    __dmul_rn(un[2], un[2])));
    x[GEX * npad + t] = __ddiv_rn(un[0], m);
    x[GEY * npad + t] = __ddiv_rn(un[1], m);
    x[GEZ * npad + t] = __ddiv_rn(un[2], m);
}

// Float-float split of the coordinates for the single-precision assembly.
__global__ void geometry32_kernel(int64_t npad, const double* __restrict__ geo, float* __restrict__ g32) {
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= npad) return;
    const int src[3] = {GX, GY, GZ};
    for (int c = 0; c < 3; ++c) {
        double v = geo[src[c] * npad + t];
        float hi = (float)v;
        g32[(2 * c) * npad + t] = hi;
        g32[(2 * c + 1) * npad + t] = (float)(v - (double)hi);
    }
    const int nsrc[3] = {GEX, GEY, GEZ}, nhi[3] = {FEX, FEY, FEZ}, nlo[3] = {FEXL, FEYL, FEZL};
    for (int c = 0; c < 3; ++c) {
        double v = geo[nsrc[c] * npad + t];
        float hi = (float)v;
        g32[nhi[c] * npad + t] = hi;
        g32[nlo[c] * npad + t] = (float)(v - (double)hi);
    }
    const double wa = geo[GWA * npad + t] * (0.25 / 3.14159265358979323846);
    const float wh = (float)wa;
    g32[FWA * npad + t] = wh;
    g32[FWAL * npad + t] = (float)(wa - (double)wh);
}

void compute_collocation(Context& ctx, Problem& p) {
    const Mesh& m = p.mesh;
    require(p.in.body_index >= 1 && p.in.body_index <= m.nbodies,
            "body_index " + std::to_string(p.in.body_index) + " out of range (mesh has " +
                std::to_string(m.nbodies) + " bodies)");
    // element list of the body in order; only linear tris/quads integrate
    std::vector<int32_t> et;
    std::vector<int64_t> en;
    for (int64_t e = 0; e < m.nelem(); ++e) {
        if (m.body[(size_t)e] != p.in.body_index) continue;
        int t = m.etype[(size_t)e];
        if (t != 5 && t != 9) continue;
        int64_t nn = m.conn_off[(size_t)e + 1] - m.conn_off[(size_t)e];
        int need = t == 5 ? 3 : 4;
        if (nn < need) throw Error(BEM_ERR_BAD_INPUT, "VTK: element " + std::to_string(e) + " has too few nodes");
        int64_t ids[4] = {0, 0, 0, 0};
        for (int a = 0; a < need; ++a) {
            ids[a] = m.conn[(size_t)(m.conn_off[(size_t)e] + a)];
            require(ids[a] >= 0 && ids[a] < m.nnodes(), "VTK: node index out of range");
        }
        et.push_back(t);
        en.insert(en.end(), ids, ids + 4);
    }
    int64_t n = (int64_t)et.size();
    require(n > 0, "body has no triangle or quad elements");
    p.n = n;
    p.geo.n = n;
    p.geo.npad = (n + 63) / 64 * 64;
    p.geo.buf.ensure(sizeof(double) * GEO_NARR * (size_t)p.geo.npad);
    // nodes, element types and connectivity staged in one grow-only buffer of
    // the context (no allocation per problem)
    const size_t b_nodes = sizeof(double) * m.nodes.size(), b_en = sizeof(int64_t) * en.size(),
                 b_et = sizeof(int32_t) * et.size();
    ctx.w_upload.ensure(b_nodes + b_en + b_et + 64);
    char* up = ctx.w_upload.as<char>();
    double* d_nodes = reinterpret_cast<double*>(up);
    int64_t* d_en = reinterpret_cast<int64_t*>(up + b_nodes);
    int32_t* d_et = reinterpret_cast<int32_t*>(up + b_nodes + b_en);
    BEM_CUDA(cudaMemcpyAsync(d_nodes, m.nodes.data(), b_nodes, cudaMemcpyHostToDevice, ctx.stream));
    BEM_CUDA(cudaMemcpyAsync(d_et, et.data(), b_et, cudaMemcpyHostToDevice, ctx.stream));
    BEM_CUDA(cudaMemcpyAsync(d_en, en.data(), b_en, cudaMemcpyHostToDevice, ctx.stream));
    int threads = 128;
    int blocks = (int)((p.geo.npad + threads - 1) / threads);
    collocation_kernel<<<blocks, threads, 0, ctx.stream>>>(n, d_nodes, d_et, d_en, p.geo.npad, p.geo.arr(0));
    BEM_CHECK_LAUNCH(&ctx);
    p.geo.buf32.ensure(sizeof(float) * GEO32_NARR * (size_t)p.geo.npad);
    geometry32_kernel<<<blocks, threads, 0, ctx.stream>>>(p.geo.npad, p.geo.arr(0), p.geo.arr32(0));
    BEM_CHECK_LAUNCH(&ctx);
    // host copy (cluster tree construction and bem_collocation)
    std::vector<double> soa((size_t)GEO_NARR * p.geo.npad);
    BEM_CUDA(cudaMemcpyAsync(soa.data(), p.geo.arr(0), sizeof(double) * soa.size(), cudaMemcpyDeviceToHost,
                             ctx.stream));
    ctx.sync();
    p.cpts.assign((size_t)n * 8, 0.0);
    for (int64_t i = 0; i < n; ++i)
        for (int k = 0; k < 8; ++k) p.cpts[(size_t)(8 * i + k)] = soa[(size_t)(k * p.geo.npad + i)];
}

void upload_field_points(Context& ctx, Problem& p) {
    p.nfp = (int64_t)p.in.field_points.size() / 3;
    p.nfp_pad = (p.nfp + 63) / 64 * 64;
    if (p.nfp_pad == 0) p.nfp_pad = 64;
    std::vector<double> soa((size_t)3 * p.nfp_pad, 0.0);
    for (int64_t i = 0; i < p.nfp; ++i)
        for (int k = 0; k < 3; ++k) soa[(size_t)(k * p.nfp_pad + i)] = p.in.field_points[(size_t)(3 * i + k)];
    p.d_fp.ensure(sizeof(double) * soa.size());
    BEM_CUDA(cudaMemcpyAsync(p.d_fp.p, soa.data(), sizeof(double) * soa.size(), cudaMemcpyHostToDevice,
                             ctx.stream));
    // float-float copy (hi, lo per coordinate) for the single-precision field kernel
    std::vector<float> ff((size_t)6 * p.nfp_pad, 0.f);
    for (int k = 0; k < 3; ++k)
        for (int64_t i = 0; i < p.nfp_pad; ++i) {
            double v = soa[(size_t)(k * p.nfp_pad + i)];
            float hi = (float)v;
            ff[(size_t)((2 * k) * p.nfp_pad + i)] = hi;
            ff[(size_t)((2 * k + 1) * p.nfp_pad + i)] = (float)(v - (double)hi);
        }
    p.d_fp32.ensure(sizeof(float) * ff.size());
    BEM_CUDA(cudaMemcpyAsync(p.d_fp32.p, ff.data(), sizeof(float) * ff.size(), cudaMemcpyHostToDevice, ctx.stream));
    ctx.sync();
}

KParams kparams(const Problem& p) {
    KParams kp;
    kp.k = p.wavenumber();
    kp.bm = p.in.method_type == 1;
    kp.beta_im = kp.bm ? 1.0 / kp.k : 0.0;   // preprocess.rs:58 beta = i/k
    kp.hdiag = p.in.problem_type == 1 ? -0.5 : 0.0;  // preprocess.rs:60-66
    kp.gdiag_im = kp.bm ? 0.5 * (1.0 / kp.k) : 0.0;  // preprocess.rs:68-74
    return kp;
}

// influence_matrix.rs:130-146
void lhs_factors(const Problem& p, cd& a, cd& b) {
    if (p.in.bc_type == 0) { a = {0, 0}; b = {1, 0}; return; }
    if (p.in.bc_type == 1) { a = {1, 0}; b = {0, 0}; return; }
    // (0, -omega rho) / Z
    double zr = p.in.bc_value[0], zi = p.in.bc_value[1];
    double nr = 0.0, ni = -p.omega() * p.in.mass_density;
    double d = zr * zr + zi * zi;
    a = {1, 0};
    b = {(nr * zr + ni * zi) / d, (ni * zr - nr * zi) / d};
}

// influence_matrix.rs:149-162
void rhs_factors(const Problem& p, cd& a, cd& b) {
    if (p.in.bc_type == 0) { a = {-1, 0}; b = {0, 0}; return; }
    if (p.in.bc_type == 1) { a = {0, 0}; b = {1, 0}; return; }
    a = {0, 0};
    b = {0, 0};
}

struct IncParams {
    double k, amp_re, amp_im, v[3], beta_im;
    int spherical, bm;
};

static IncParams inc_params(const Problem& p) {
    IncParams q;
    q.k = p.wavenumber();
    // amp = p_amp / (i omega rho)
    double den = p.omega() * p.in.mass_density;
    double ar = p.in.incident_amp[0], ai = p.in.incident_amp[1];
    // (ar + i ai) / (0 + i den) = (ai den)/den^2 + i(-ar den)/den^2
    q.amp_re = (ar * 0.0 + ai * den) / (den * den);
    q.amp_im = (ai * 0.0 - ar * den) / (den * den);
    double nv = std::sqrt(p.in.incident_vec[0] * p.in.incident_vec[0] + p.in.incident_vec[1] * p.in.incident_vec[1] +
                          p.in.incident_vec[2] * p.in.incident_vec[2]);
    for (int k = 0; k < 3; ++k) q.v[k] = p.in.incident_vec[k] / nv;  // direction / origin normalised
    q.spherical = p.in.incident_type == 1;
    q.bm = p.in.method_type == 1;
    q.beta_im = q.bm ? 1.0 / q.k : 0.0;
    return q;
}

// incident_wave.rs:7-63 (surface, with the Burton-Miller term) and :66-99
// (field points, no normal): the value at point i of pts (x y z, then the
// normal, arrays `stride` apart).
__device__ __forceinline__ z2 incident_value(int64_t i, int64_t stride, const double* __restrict__ pts,
                                             const IncParams& q, int with_normal) {
    double x = pts[i], y = pts[stride + i], z = pts[2 * stride + i];
    z2 amp = {q.amp_re, q.amp_im};
    z2 val;
    if (!q.spherical) {
        double a = q.k * (q.v[0] * x + q.v[1] * y + q.v[2] * z);
        double s, c;
        sincos(a, &s, &c);
        z2 phi = cmul(amp, z2{c, s});
        val = phi;
        if (with_normal && q.bm) {
            double dn = q.v[0] * pts[3 * stride + i] + q.v[1] * pts[4 * stride + i] + q.v[2] * pts[5 * stride + i];
            z2 vn = cscale(cmul(phi, z2{0.0, q.k}), dn);
            val = cadd(val, cmul(z2{0.0, q.beta_im}, vn));
        }
    } else {
        double rx = x - q.v[0], ry = y - q.v[1], rz = z - q.v[2];
        double r = sqrt(rx * rx + ry * ry + rz * rz);
        double s, c;
        sincos(q.k * r, &s, &c);
        z2 ph = cmul(amp, z2{c, s});
        double den = 4.0 * 3.14159265358979323846 * r;
        z2 phi = {ph.x / den, ph.y / den};
        val = phi;
        if (with_normal && q.bm) {
            double dn = (rx / r) * pts[3 * stride + i] + (ry / r) * pts[4 * stride + i] + (rz / r) * pts[5 * stride + i];
            z2 vn = cscale(cmul(phi, z2{-1.0 / r, q.k}), dn);
            val = cadd(val, cmul(z2{0.0, q.beta_im}, vn));
        }
    }
    return val;
}

__global__ void incident_kernel(int64_t n, int64_t stride, const double* __restrict__ pts, IncParams q,
                                int with_normal, double2* __restrict__ out) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = incident_value(i, stride, pts, q, with_normal);
}

// Several systems in one launch: a flattened grid of 128-point blocks, the
// job of a block found by bisection on blk0.  Surface jobs also form the
// GMRES right-hand side out2 = s inc + bc rowsum (solve.rs:35-69).
struct IncJob {
    const double* pts;
    int64_t n, stride, blk0;
    IncParams q;
    int with_normal, pad;
    double sgn;
    double2 bc;
    const double2* rowsum;
    double2* out;   // the incident values
    double2* out2;  // the right-hand side (surface jobs; may be null)
};

__global__ void incident_batch_kernel(const IncJob* __restrict__ jobs, int njobs) {
    const int64_t b = blockIdx.x;
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (jobs[mid].blk0 <= b) lo = mid;
        else hi = mid - 1;
    }
    const IncJob& J = jobs[lo];
    const int64_t i = (b - J.blk0) * 128 + threadIdx.x;
    if (i >= J.n) return;
    const z2 v = incident_value(i, J.stride, J.pts, J.q, J.with_normal);
    J.out[i] = v;
    if (J.out2) {
        double2 r = cscale(v, J.sgn);
        if (J.rowsum) cfma(r, J.bc, J.rowsum[i]);
        J.out2[i] = r;
    }
}

void incident_surface(Context& ctx, const Problem& p, double2* out) {
    IncParams q = inc_params(p);
    int threads = 128;
    int blocks = (int)((p.n + threads - 1) / threads);
    incident_kernel<<<blocks, threads, 0, ctx.stream>>>(p.n, p.geo.npad, p.geo.arr(0), q, 1, out);
    BEM_CHECK_LAUNCH(&ctx);
}

void incident_batch(Context& ctx, const std::vector<IncItem>& items) {
    if (items.empty()) return;
    std::vector<IncJob> jobs;
    int64_t blk = 0;
    for (const IncItem& it : items) {
        Problem& p = const_cast<Problem&>(*it.p);
        const int64_t f0 = p.ifreq;
        p.ifreq = it.ifreq;
        p.select_rhs(it.rhs);
        IncJob J{};
        J.q = inc_params(p);
        p.select_rhs(0);
        p.ifreq = f0;
        J.with_normal = it.field ? 0 : 1;
        J.pts = it.field ? p.d_fp.as<double>() : p.geo.arr(0);
        J.n = it.field ? p.nfp : p.n;
        J.stride = it.field ? p.nfp_pad : p.geo.npad;
        J.blk0 = blk;
        J.sgn = it.sgn;
        J.bc = make_double2(it.bc.re, it.bc.im);
        J.rowsum = it.rowsum;
        J.out = it.out;
        J.out2 = it.rhs_out;
        if (J.n == 0) continue;
        blk += (J.n + 127) / 128;
        jobs.push_back(J);
    }
    if (jobs.empty()) return;
    DevBuf d;
    d.ensure(sizeof(IncJob) * jobs.size());
    BEM_CUDA(cudaMemcpyAsync(d.p, jobs.data(), sizeof(IncJob) * jobs.size(), cudaMemcpyHostToDevice, ctx.stream));
    incident_batch_kernel<<<(unsigned)blk, 128, 0, ctx.stream>>>(d.as<IncJob>(), (int)jobs.size());
    BEM_CHECK_LAUNCH(&ctx);
    ctx.sync();  // the job list is freed on return
}

void incident_field(Context& ctx, const Problem& p, double2* out) {
    if (p.nfp == 0) return;
    IncParams q = inc_params(p);
    int threads = 128;
    int blocks = (int)((p.nfp + threads - 1) / threads);
    incident_kernel<<<blocks, threads, 0, ctx.stream>>>(p.nfp, p.nfp_pad, p.d_fp.as<double>(), q, 0, out);
    BEM_CHECK_LAUNCH(&ctx);
}

}  // namespace bem
