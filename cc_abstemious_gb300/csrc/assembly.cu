// Influence-matrix assembly (influence_matrix.rs:12-230) and field evaluation
// (influence_matrix.rs:101-127, solve.rs:173-185) on sm_103a.
//
// Layout: matrices are column-major complex (double2 / float2) with leading
// dimension ld; row i is the collocation (observation) point, column j the
// source element.  A CTA owns a 64 x 64 tile: the geometry of its 64 rows and
// 64 columns is staged into shared memory by bulk asynchronous copies (TMA)
// completed on an mbarrier, and each warp stores 32 consecutive rows of one
// column (512 contiguous bytes per matrix for FP64).
#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "complex.cuh"
#include "tma.cuh"
#include "kernels.cuh"

namespace bem {

// influence_matrix.rs:12-37.  (x, e_x): source point and its normal; (y, e_y):
// observation point and its normal.  Returns g and h without the wt*area scale.
__device__ __forceinline__ void greens64(double k, int bm, double beta_im, double xx, double xy, double xz,
                                         double exx, double exy, double exz, double yx, double yy, double yz,
                                         double eyx, double eyy, double eyz, z2& g, z2& h) {
    double rx = xx - yx, ry = xy - yy, rz = xz - yz;
    double r = sqrt(rx * rx + ry * ry + rz * rz);
    double inv = 1.0 / r;
    double erx = rx * inv, ery = ry * inv, erz = rz * inv;
    double s, c;
    sincos(k * r, &s, &c);
    double q = inv * (1.0 / (4.0 * PI_D));
    g = make_double2(c * q, s * q);
    z2 f1 = make_double2(-inv, k);
    double rdoty = erx * eyx + ery * eyy + erz * eyz;
    z2 gf1 = cmul(g, f1);
    h = cscale(gf1, -rdoty);
    if (bm) {
        double rdotx = erx * exx + ery * exy + erz * exz;
        double nxy = eyx * exx + eyy * exy + eyz * exz;
        z2 dg = cscale(gf1, rdotx);
        z2 t1 = cscale(cneg(f1), nxy);
        z2 t2 = cscale(cscale(make_double2(k * k * r + 3.0 * f1.x, 3.0 * f1.y), rdotx), rdoty);
        z2 dh = cmul(cscale(g, inv), csub(t1, t2));
        // beta = i * beta_im
        g = cadd(g, make_double2(-beta_im * dg.y, beta_im * dg.x));
        h = cadd(h, make_double2(-beta_im * dh.y, beta_im * dh.x));
    }
}

struct TileGeo64 {
    // columns: x y z ex ey ez wa area wt ; rows: x y z ex ey ez
    double cx[TILE], cy[TILE], cz[TILE], cex[TILE], cey[TILE], cez[TILE], cwa[TILE], carea[TILE], cwt[TILE];
    double rx[TILE], ry[TILE], rz[TILE], rex[TILE], rey[TILE], rez[TILE];
};

// Stage the tile geometry with bulk copies; returns false on a timed-out wait.
__device__ __forceinline__ bool stage_tile64(TileGeo64& t, uint64_t* bar, const double* geo, int64_t npad,
                                             int64_t I0, int64_t J0) {
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    const uint32_t B = TILE * sizeof(double);
    if (threadIdx.x == 0) {
        mbar_arrive_expect_tx(bar, 15 * B);
        const int csrc[9] = {GX, GY, GZ, GEX, GEY, GEZ, GWA, GAREA, GWT};
        double* cdst[9] = {t.cx, t.cy, t.cz, t.cex, t.cey, t.cez, t.cwa, t.carea, t.cwt};
        for (int a = 0; a < 9; ++a) bulk_g2s(cdst[a], geo + csrc[a] * npad + J0, B, bar);
        const int rsrc[6] = {GX, GY, GZ, GEX, GEY, GEZ};
        double* rdst[6] = {t.rx, t.ry, t.rz, t.rex, t.rey, t.rez};
        for (int a = 0; a < 6; ++a) bulk_g2s(rdst[a], geo + rsrc[a] * npad + I0, B, bar);
    }
    return mbar_wait_bounded(bar, 0);
}

// MODE 0: write H and G (get_dense_surface_matrices).
// MODE 1: write A = alpha H + beta G; optional per-column-tile partial row sums
//         of gamma H + delta G (the uniform-BC right-hand side of solve.rs:35-69).
template <int MODE>
__global__ void __launch_bounds__(ASM_THREADS) assemble64_kernel(
    int64_t n, int64_t npad, const double* __restrict__ geo, KParams kp, double2* __restrict__ H,
    double2* __restrict__ G, int64_t ld, z2 alpha, z2 beta, z2 gamma, z2 delta, double2* __restrict__ part,
    int* __restrict__ err) {
    __shared__ __align__(128) TileGeo64 t;
    __shared__ __align__(8) uint64_t bar;
    __shared__ z2 red[ASM_THREADS];
    const int64_t I0 = (int64_t)blockIdx.y * TILE, J0 = (int64_t)blockIdx.x * TILE;
    if (!stage_tile64(t, &bar, geo, npad, I0, J0)) {
        if (threadIdx.x == 0) atomicOr(err, DEVERR_MBAR_TIMEOUT);
        mbar_wait_bounded(&bar, 0);
        return;
    }
    const int tx = threadIdx.x & (TILE - 1), ty = threadIdx.x >> 6;
    const int64_t i = I0 + tx;
    const double yx = t.rx[tx], yy = t.ry[tx], yz = t.rz[tx];
    const double eyx = t.rex[tx], eyy = t.rey[tx], eyz = t.rez[tx];
    z2 acc = make_double2(0.0, 0.0);
#pragma unroll 1
    for (int c = 0; c < TILE / 4; ++c) {
        const int jj = ty + 4 * c;
        const int64_t j = J0 + jj;
        z2 g, h;
        if (i == j) {
            self_term64(t.carea[jj], t.cwt[jj], kp.bm, kp.beta_im, kp.hdiag, kp.gdiag_im, g, h);
        } else {
            greens64(kp.k, kp.bm, kp.beta_im, t.cx[jj], t.cy[jj], t.cz[jj], t.cex[jj], t.cey[jj], t.cez[jj], yx, yy,
                     yz, eyx, eyy, eyz, g, h);
            double wa = t.cwa[jj];
            g = cscale(g, wa);
            h = cscale(h, wa);
        }
        if (i < n && j < n) {
            if (MODE == 0) {
                H[j * ld + i] = h;
                G[j * ld + i] = g;
            } else {
                z2 a = cmul(alpha, h);
                cfma(a, beta, g);
                H[j * ld + i] = a;
                if (part) {
                    cfma(acc, gamma, h);
                    cfma(acc, delta, g);
                }
            }
        }
    }
    if (MODE == 1 && part) {
        red[threadIdx.x] = acc;
        __syncthreads();
        if (ty == 0 && i < n) {
            z2 s = red[tx];
            for (int q = 1; q < 4; ++q) s = cadd(s, red[tx + TILE * q]);
            part[(int64_t)blockIdx.x * npad + i] = s;
        }
    }
}

// rowsum[i] = sum over column tiles of part[t][i] (fixed order).
__global__ void reduce_parts_kernel(int64_t n, int64_t npad, int ntiles, const double2* __restrict__ part,
                                    double2* __restrict__ out) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    z2 s = make_double2(0.0, 0.0);
    for (int t = 0; t < ntiles; ++t) s = cadd(s, part[(int64_t)t * npad + i]);
    out[i] = s;
}

int* device_err(Context& ctx) {
    ctx.w_flags.ensure(256);
    return ctx.w_flags.as<int>();
}

void check_device_err(Context& ctx) {
    int h = 0;
    BEM_CUDA(cudaMemcpyAsync(&h, ctx.w_flags.p, sizeof(int), cudaMemcpyDeviceToHost, ctx.stream));
    ctx.sync();
    if (h) {
        BEM_CUDA(cudaMemsetAsync(ctx.w_flags.p, 0, sizeof(int), ctx.stream));
        throw Error(BEM_ERR_TIMEOUT, "a bounded device-side wait gave up (code " + std::to_string(h) + ")");
    }
}

void launch_reduce_parts(Context& ctx, int64_t n, int64_t npad, int ntiles, const double2* part, double2* out) {
    reduce_parts_kernel<<<(unsigned)((n + 255) / 256), 256, 0, ctx.stream>>>(n, npad, ntiles, part, out);
    BEM_CHECK_LAUNCH(&ctx);
}

void assemble_surface_fp64(Context& ctx, const Problem& p, double2* H, double2* G, int64_t ld) {
    int* err = device_err(ctx);
    BEM_CUDA(cudaMemsetAsync(err, 0, sizeof(int), ctx.stream));
    dim3 grid((unsigned)(p.geo.npad / TILE), (unsigned)(p.geo.npad / TILE));
    z2 zero = make_double2(0, 0);
    assemble64_kernel<0><<<grid, ASM_THREADS, 0, ctx.stream>>>(p.n, p.geo.npad, p.geo.arr(0), kparams(p), H, G, ld,
                                                              zero, zero, zero, zero, nullptr, err);
    BEM_CHECK_LAUNCH(&ctx);
    check_device_err(ctx);
}

void assemble_system_fp64(Context& ctx, const Problem& p, double2* A, int64_t ld, cd alpha, cd beta, cd gamma,
                          cd delta, double2* rowsum) {
    int* err = device_err(ctx);
    BEM_CUDA(cudaMemsetAsync(err, 0, sizeof(int), ctx.stream));
    int ntiles = (int)(p.geo.npad / TILE);
    double2* part = nullptr;
    if (rowsum) {
        ctx.w_part.ensure(sizeof(double2) * (size_t)ntiles * p.geo.npad);
        part = ctx.w_part.as<double2>();
    }
    dim3 grid((unsigned)ntiles, (unsigned)ntiles);
    assemble64_kernel<1><<<grid, ASM_THREADS, 0, ctx.stream>>>(
        p.n, p.geo.npad, p.geo.arr(0), kparams(p), A, nullptr, ld, make_double2(alpha.re, alpha.im),
        make_double2(beta.re, beta.im), make_double2(gamma.re, gamma.im), make_double2(delta.re, delta.im), part, err);
    BEM_CHECK_LAUNCH(&ctx);
    if (rowsum) {
        reduce_parts_kernel<<<(unsigned)((p.n + 255) / 256), 256, 0, ctx.stream>>>(p.n, p.geo.npad, ntiles, part,
                                                                                    rowsum);
        BEM_CHECK_LAUNCH(&ctx);
    }
    check_device_err(ctx);
}

// ---------------------------------------------------------------------------
// influence_matrix.rs:170-230: row i over columns J, or column j over rows I,
// of alpha H + beta G including hdiag/gdiag at the first diagonal position.
__global__ void row_or_column_kernel(int64_t npad, const double* __restrict__ geo, KParams kp,
                                     const int64_t* __restrict__ I, int64_t ni, const int64_t* __restrict__ J,
                                     int64_t nj, z2 alpha, z2 beta, int64_t diag_pos, double2* __restrict__ out) {
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int64_t len = ni == 1 ? nj : ni;
    if (t >= len) return;
    int64_t i = ni == 1 ? I[0] : I[t];
    int64_t j = ni == 1 ? J[t] : J[0];
    z2 g, h;
    if (i == j) {
        self_term64(geo[GAREA * npad + j], geo[GWT * npad + j], kp.bm, kp.beta_im, 0.0, 0.0, g, h);
        if (t == diag_pos) {
            h.x += kp.hdiag;
            g.y += kp.gdiag_im;
        }
    } else {
        greens64(kp.k, kp.bm, kp.beta_im, geo[GX * npad + j], geo[GY * npad + j], geo[GZ * npad + j],
                 geo[GEX * npad + j], geo[GEY * npad + j], geo[GEZ * npad + j], geo[GX * npad + i], geo[GY * npad + i],
                 geo[GZ * npad + i], geo[GEX * npad + i], geo[GEY * npad + i], geo[GEZ * npad + i], g, h);
        double wa = geo[GWA * npad + j];
        g = cscale(g, wa);
        h = cscale(h, wa);
    }
    z2 a = cmul(beta, g);
    cfma(a, alpha, h);
    out[t] = a;
}

void row_or_column(Context& ctx, const Problem& p, const int64_t* dI, int64_t ni, const int64_t* dJ, int64_t nj,
                   int side, double2* out, int64_t diag_pos) {
    cd a, b;
    if (side) lhs_factors(p, a, b); else rhs_factors(p, a, b);
    int64_t len = ni == 1 ? nj : ni;
    if (len == 0) return;
    row_or_column_kernel<<<(unsigned)((len + 127) / 128), 128, 0, ctx.stream>>>(
        p.geo.npad, p.geo.arr(0), kparams(p), dI, ni, dJ, nj, make_double2(a.re, a.im), make_double2(b.re, b.im),
        diag_pos, out);
    BEM_CHECK_LAUNCH(&ctx);
}

// ---------------------------------------------------------------------------
// Field matrices (influence_matrix.rs:101-127): classical kernel, the field
// point as x and the element as y with its normal.  M, L are nfp x n.
__global__ void field_matrices_kernel(int64_t nfp, int64_t fpad, const double* __restrict__ fp, int64_t n,
                                      int64_t npad, const double* __restrict__ geo, double k,
                                      double2* __restrict__ M, double2* __restrict__ L, int64_t ld) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int64_t j = blockIdx.y;
    if (i >= nfp) return;
    z2 g, h;
    greens64(k, 0, 0.0, fp[i], fp[fpad + i], fp[2 * fpad + i], 0, 0, 0, geo[GX * npad + j], geo[GY * npad + j],
             geo[GZ * npad + j], geo[GEX * npad + j], geo[GEY * npad + j], geo[GEZ * npad + j], g, h);
    double wa = geo[GWA * npad + j];
    M[j * ld + i] = cscale(h, wa);
    L[j * ld + i] = cscale(g, wa);
}

void field_matrices_fp64(Context& ctx, const Problem& p, double2* M, double2* L, int64_t ld) {
    if (p.nfp == 0) return;
    dim3 grid((unsigned)((p.nfp + 127) / 128), (unsigned)p.n);
    field_matrices_kernel<<<grid, 128, 0, ctx.stream>>>(p.nfp, p.nfp_pad, p.d_fp.as<double>(), p.n, p.geo.npad,
                                                       p.geo.arr(0), p.wavenumber(), M, L, ld);
    BEM_CHECK_LAUNCH(&ctx);
}

// Fused field evaluation: out_i = [inc_i] - sum_j M_ij phi_j + sum_j L_ij vn_j
// without storing M and L.  One CTA per field point, fixed-order reduction.
constexpr int FIELD_THREADS = 256;
__global__ void __launch_bounds__(FIELD_THREADS) evaluate_field_kernel(
    int64_t nfp, int64_t fpad, const double* __restrict__ fp, int64_t n, int64_t npad,
    const double* __restrict__ geo, double k, const double2* __restrict__ phi, const double2* __restrict__ vn,
    const double2* __restrict__ inc, double2* __restrict__ out) {
    __shared__ z2 red[FIELD_THREADS];
    int64_t i = blockIdx.x;
    double px = fp[i], py = fp[fpad + i], pz = fp[2 * fpad + i];
    z2 acc = make_double2(0, 0);
    for (int64_t j = threadIdx.x; j < n; j += FIELD_THREADS) {
        z2 g, h;
        greens64(k, 0, 0.0, px, py, pz, 0, 0, 0, geo[GX * npad + j], geo[GY * npad + j], geo[GZ * npad + j],
                 geo[GEX * npad + j], geo[GEY * npad + j], geo[GEZ * npad + j], g, h);
        double wa = geo[GWA * npad + j];
        cfma(acc, cscale(h, -wa), phi[j]);
        cfma(acc, cscale(g, wa), vn[j]);
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = FIELD_THREADS / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] = cadd(red[threadIdx.x], red[threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x == 0) out[i] = inc ? cadd(inc[i], red[0]) : red[0];
}

void evaluate_field(Context& ctx, const Problem& p, const double2* phi, const double2* vn, const double2* inc,
                    double2* out) {
    if (p.nfp == 0) return;
    evaluate_field_kernel<<<(unsigned)p.nfp, FIELD_THREADS, 0, ctx.stream>>>(
        p.nfp, p.nfp_pad, p.d_fp.as<double>(), p.n, p.geo.npad, p.geo.arr(0), p.wavenumber(), phi, vn, inc, out);
    BEM_CHECK_LAUNCH(&ctx);
}

}  // namespace bem
