// Hierarchical matrices (h_matrix.rs, aca.rs, cluster.rs, block.rs).
//
// Device: the geometric cluster tree and the block tree with its flattened
// leaf list (tree.cu), then every leaf block is filled in one batched pass -- inadmissible
// leaves as dense FP64 blocks, admissible leaves by adaptive cross
// approximation (one CTA per leaf running the reference's partially pivoted
// ACA with the rand 0.9 StdRng pivot stream restated below), followed by the
// QR + SVD recompression, also one CTA per leaf.  The mat-vec multiplies every
// leaf in parallel into a per-leaf output slice, then reduces each global row
// over its leaves in a fixed order (deterministic).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <memory>

#include "common.cuh"
#include "complex.cuh"
#include "gmres.cuh"
#include "hmatrix.cuh"
#include "kernels.cuh"
#include "mixed.cuh"
#include "tree.cuh"

struct bem_hmatrix {
    bem::HMatrixDev* h;
    bem_ctx* ctx;
};

namespace bem {

// Leaf descriptor shared with the kernels.
struct HLeaf {
    int64_t row_off, m;   // into rows[]
    int64_t col_off, n;   // into cols[]
    int64_t store_off;    // dense: m*n entries; admissible: U (m*kmax) then V (n*kmax)
    int64_t scratch_off;  // ACA scratch: 2(m+n) complex + flags
    int64_t y_off;        // mat-vec output slice (m entries)
    int32_t adm, kmax;
    int32_t rank, pad;
    double norm;
};

struct HMatrixDev {
    int64_t n = 0;
    double norm = 0;
    std::vector<HLeaf> leaves;
    std::vector<int64_t> rows, cols;
    DevBuf d_leaves, d_rows, d_cols, d_store, d_scratch, d_y, d_rowptr, d_rowent, d_vec;
    int64_t nadm = 0, ninadm = 0, stored = 0, rank_sum = 0;
};

// ---------------------------------------------------------------------------
// Entry (i, j) of alpha H + beta G (influence_matrix.rs:170-230 restated per
// entry; column lists hold distinct indices so the diagonal appears once).
struct GenParams {
    KParams kp;
    z2 alpha, beta;
    int64_t npad;
    const double* geo;
};

__device__ __forceinline__ z2 gen_entry(const GenParams& g, int64_t i, int64_t j) {
    const double* geo = g.geo;
    const int64_t np = g.npad;
    z2 gg, hh;
    if (i == j) {
        self_term64(geo[GAREA * np + j], geo[GWT * np + j], g.kp.bm, g.kp.beta_im, g.kp.hdiag, g.kp.gdiag_im, gg, hh);
    } else {
        // source x = element j, observation y = collocation point i
        double rx = geo[GX * np + j] - geo[GX * np + i], ry = geo[GY * np + j] - geo[GY * np + i],
               rz = geo[GZ * np + j] - geo[GZ * np + i];
        double r = sqrt(rx * rx + ry * ry + rz * rz);
        double inv = 1.0 / r;
        double erx = rx * inv, ery = ry * inv, erz = rz * inv;
        double s, c;
        sincos(g.kp.k * r, &s, &c);
        double q = inv * (1.0 / (4.0 * PI_D));
        gg = make_double2(c * q, s * q);
        z2 f1 = make_double2(-inv, g.kp.k);
        double eyx = geo[GEX * np + i], eyy = geo[GEY * np + i], eyz = geo[GEZ * np + i];
        double rdoty = erx * eyx + ery * eyy + erz * eyz;
        z2 gf1 = cmul(gg, f1);
        hh = cscale(gf1, -rdoty);
        if (g.kp.bm) {
            double exx = geo[GEX * np + j], exy = geo[GEY * np + j], exz = geo[GEZ * np + j];
            double rdotx = erx * exx + ery * exy + erz * exz;
            double nxy = eyx * exx + eyy * exy + eyz * exz;
            z2 dg = cscale(gf1, rdotx);
            z2 t1 = cscale(cneg(f1), nxy);
            z2 t2 = cscale(cscale(make_double2(g.kp.k * g.kp.k * r + 3.0 * f1.x, 3.0 * f1.y), rdotx), rdoty);
            z2 dh = cmul(cscale(gg, inv), csub(t1, t2));
            gg = cadd(gg, make_double2(-g.kp.beta_im * dg.y, g.kp.beta_im * dg.x));
            hh = cadd(hh, make_double2(-g.kp.beta_im * dh.y, g.kp.beta_im * dh.x));
        }
        double wa = geo[GWA * np + j];
        gg = cscale(gg, wa);
        hh = cscale(hh, wa);
    }
    z2 a = cmul(g.beta, gg);
    cfma(a, g.alpha, hh);
    return a;
}

// ---------------------------------------------------------------------------
// rand 0.9 StdRng (ChaCha12, rand_core seed_from_u64 via PCG32) and
// UniformUsize sampling of ranges below 2^32 -- the ACA pivot stream of
// aca.rs:64-68, evaluated by one thread.
struct DevRng {
    uint32_t key[8];
    uint64_t counter;
    uint32_t buf[16];
    int idx;
};

__device__ __forceinline__ uint32_t rotl32d(uint32_t v, int c) { return (v << c) | (v >> (32 - c)); }

__device__ void chacha12_block_dev(const uint32_t* key, uint64_t ctr, uint32_t* out) {
    uint32_t st[16] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u, key[0], key[1], key[2], key[3],
                       key[4], key[5], key[6], key[7], (uint32_t)ctr, (uint32_t)(ctr >> 32), 0u, 0u};
    uint32_t s[16];
    for (int i = 0; i < 16; ++i) s[i] = st[i];
#define DQR(a, b, c, d)                                   \
    s[a] += s[b]; s[d] = rotl32d(s[d] ^ s[a], 16);        \
    s[c] += s[d]; s[b] = rotl32d(s[b] ^ s[c], 12);        \
    s[a] += s[b]; s[d] = rotl32d(s[d] ^ s[a], 8);         \
    s[c] += s[d]; s[b] = rotl32d(s[b] ^ s[c], 7);
    for (int r = 0; r < 6; ++r) {
        DQR(0, 4, 8, 12) DQR(1, 5, 9, 13) DQR(2, 6, 10, 14) DQR(3, 7, 11, 15)
        DQR(0, 5, 10, 15) DQR(1, 6, 11, 12) DQR(2, 7, 8, 13) DQR(3, 4, 9, 14)
    }
#undef DQR
    for (int i = 0; i < 16; ++i) out[i] = s[i] + st[i];
}

// Words are consumed in block order; the reference buffers four blocks at a
// time, which yields the same stream.
__device__ void rng_seed(DevRng& r, uint64_t state) {
    for (int i = 0; i < 8; ++i) {
        state = state * 6364136223846793005ull + 11634580027462260723ull;
        uint32_t xs = (uint32_t)(((state >> 18) ^ state) >> 27);
        uint32_t rot = (uint32_t)(state >> 59);
        r.key[i] = (xs >> rot) | (xs << ((32 - rot) & 31));
    }
    r.counter = 0;
    r.idx = 16;
}

__device__ uint32_t rng_u32(DevRng& r) {
    if (r.idx >= 16) {
        chacha12_block_dev(r.key, r.counter, r.buf);
        r.counter += 1;
        r.idx = 0;
    }
    return r.buf[r.idx++];
}

__device__ int64_t rng_uniform_incl(DevRng& r, uint32_t hi) {
    uint32_t range = hi + 1u;
    if (range == 0) return (int64_t)rng_u32(r);
    uint32_t thresh = (0u - range) % range;
    for (int guard = 0; guard < 1 << 20; ++guard) {
        uint64_t m = (uint64_t)rng_u32(r) * range;
        if ((uint32_t)m >= thresh) return (int64_t)(m >> 32);
    }
    return 0;
}

// ---------------------------------------------------------------------------
// Block-level reductions for the leaf kernels (blockDim multiple of 32, <= 1024).
__device__ __forceinline__ double bsum(double v, double* sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    if (w == 0) {
        v = l < (int)(blockDim.x >> 5) ? sh[l] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (l == 0) sh[40] = v;
    }
    __syncthreads();
    return sh[40];
}

__device__ __forceinline__ z2 bsum2(z2 v, double* sh) {
    double a = bsum(v.x, sh);
    double b = bsum(v.y, sh);
    return make_double2(a, b);
}

// Sum of a complex value over the 32 lanes of a warp (every lane gets it).
__device__ __forceinline__ z2 wsum2(z2 v) {
    for (int o = 16; o > 0; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
    }
    return v;
}

__device__ __forceinline__ double wsum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// argmax of |v[t]| over t not excluded; first index wins ties (aca.rs:256-268).
__device__ int64_t bargmax_excl(const double2* v, const int8_t* excl, int64_t len, double* sh, int64_t* shi) {
    double best = -1.0;
    int64_t bi = len;
    for (int64_t t = threadIdx.x; t < len; t += blockDim.x) {
        if (excl[t]) continue;
        double a = hypot(v[t].x, v[t].y);
        if (best < a) { best = a; bi = t; }
    }
    for (int o = 16; o > 0; o >>= 1) {
        double ob = __shfl_down_sync(0xffffffffu, best, o);
        int64_t oi = __shfl_down_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
    }
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) { sh[w] = best; shi[w] = bi; }
    __syncthreads();
    if (w == 0) {
        int nw = blockDim.x >> 5;
        best = l < nw ? sh[l] : -1.0;
        bi = l < nw ? shi[l] : len;
        for (int o = 16; o > 0; o >>= 1) {
            double ob = __shfl_down_sync(0xffffffffu, best, o);
            int64_t oi = __shfl_down_sync(0xffffffffu, bi, o);
            if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
        }
        if (l == 0) shi[32] = bi;
    }
    __syncthreads();
    return shi[32];
}

constexpr int LEAF_THREADS = 256;

// Dense (inadmissible) leaves: one CTA per leaf, entries column-major m x n.
__global__ void __launch_bounds__(LEAF_THREADS) hm_dense_fill_kernel(const HLeaf* __restrict__ leaves,
                                                                     const int32_t* __restrict__ list,
                                                                     const int64_t* __restrict__ rows,
                                                                     const int64_t* __restrict__ cols, GenParams g,
                                                                     double2* __restrict__ store) {
    const HLeaf L = leaves[list[blockIdx.x]];
    double2* D = store + L.store_off;
    for (int64_t t = threadIdx.x; t < L.m * L.n; t += blockDim.x) {
        int64_t jj = t / L.m, ii = t - jj * L.m;
        D[t] = gen_entry(g, rows[L.row_off + ii], cols[L.col_off + jj]);
    }
}

// Residual row i (local) of the current approximation: A[i, :] - sum_k u_k[i] v_k.
__device__ void aca_res_row(const GenParams& g, const HLeaf& L, const int64_t* rows, const int64_t* cols,
                            const double2* U, const double2* V, int rank, int64_t i, double2* out) {
    const int64_t gi = rows[L.row_off + i];
    for (int64_t j = threadIdx.x; j < L.n; j += blockDim.x) {
        z2 a = gen_entry(g, gi, cols[L.col_off + j]);
        for (int k = 0; k < rank; ++k) cfma(a, cneg(U[(size_t)k * L.m + i]), V[(size_t)k * L.n + j]);
        out[j] = a;
    }
    __syncthreads();
}

__device__ void aca_res_col(const GenParams& g, const HLeaf& L, const int64_t* rows, const int64_t* cols,
                            const double2* U, const double2* V, int rank, int64_t j, double2* out) {
    const int64_t gj = cols[L.col_off + j];
    for (int64_t i = threadIdx.x; i < L.m; i += blockDim.x) {
        z2 a = gen_entry(g, rows[L.row_off + i], gj);
        for (int k = 0; k < rank; ++k) cfma(a, cneg(V[(size_t)k * L.n + j]), U[(size_t)k * L.m + i]);
        out[i] = a;
    }
    __syncthreads();
}

__device__ __forceinline__ double bnsq(const double2* a, int64_t len, double* sh) {
    double acc = 0;
    for (int64_t t = threadIdx.x; t < len; t += blockDim.x) acc += a[t].x * a[t].x + a[t].y * a[t].y;
    return bsum(acc, sh);
}

// Partially pivoted ACA (aca.rs:57-136) of every admissible leaf.
__global__ void __launch_bounds__(LEAF_THREADS) hm_aca_kernel(HLeaf* __restrict__ leaves,
                                                              const int32_t* __restrict__ list,
                                                              const int64_t* __restrict__ rows,
                                                              const int64_t* __restrict__ cols, GenParams g,
                                                              double2* __restrict__ store, double2* __restrict__ scr,
                                                              double tol, int* __restrict__ err) {
    __shared__ double sh[48];
    __shared__ int64_t shi[33];
    __shared__ DevRng rng;
    __shared__ int64_t s_iref, s_jref, s_istar, s_jstar;
    __shared__ double s_total;
    __shared__ int s_stop;
    __shared__ double s_prod[256];  // one per earlier rank (kmax <= ACA_RMAX = 256)
    HLeaf& L = leaves[list[blockIdx.x]];
    const int64_t m = L.m, n = L.n;
    const int64_t nr = m < n ? m : n;
    double2* U = store + L.store_off;
    double2* V = U + (size_t)m * L.kmax;
    double2* riref = scr + L.scratch_off;
    double2* rjref = riref + n;
    double2* ristar = rjref + m;
    double2* rjstar = ristar + n;
    int8_t* iex = reinterpret_cast<int8_t*>(rjstar + m);
    int8_t* jex = iex + m;
    for (int64_t t = threadIdx.x; t < m; t += blockDim.x) iex[t] = 0;
    for (int64_t t = threadIdx.x; t < n; t += blockDim.x) jex[t] = 0;
    if (threadIdx.x == 0) {
        rng_seed(rng, 10);
        s_iref = rng_uniform_incl(rng, (uint32_t)(nr - 1));
        s_jref = rng_uniform_incl(rng, (uint32_t)(nr - 1));
        s_total = 0;
        s_stop = 0;
    }
    __syncthreads();
    aca_res_row(g, L, rows, cols, U, V, 0, s_iref, riref);
    aca_res_col(g, L, rows, cols, U, V, 0, s_jref, rjref);
    int rank = 0;
    for (int64_t k = 0; k < nr; ++k) {
        if (k >= L.kmax) {  // rank cap of the storage reached before the stopping test
            if (threadIdx.x == 0) atomicOr(err, 8);
            break;
        }
        int64_t jstar = bargmax_excl(riref, jex, n, sh, shi);
        double jval = hypot(riref[jstar].x, riref[jstar].y);
        int64_t istar = bargmax_excl(rjref, iex, m, sh, shi);
        double ival = hypot(rjref[istar].x, rjref[istar].y);
        if (ival > jval) {
            aca_res_row(g, L, rows, cols, U, V, rank, istar, ristar);
            jstar = bargmax_excl(ristar, jex, n, sh, shi);
            aca_res_col(g, L, rows, cols, U, V, rank, jstar, rjstar);
        } else {
            aca_res_col(g, L, rows, cols, U, V, rank, jstar, rjstar);
            istar = bargmax_excl(rjstar, iex, m, sh, shi);
            aca_res_row(g, L, rows, cols, U, V, rank, istar, ristar);
        }
        const z2 piv = ristar[jstar];
        __syncthreads();
        if (threadIdx.x == 0) {
            iex[istar] = 1;
            jex[jstar] = 1;
        }
        const z2 f = cdiv(make_double2(1.0, 0.0), piv);
        double2* uk = U + (size_t)k * m;
        double2* vk = V + (size_t)k * n;
        for (int64_t t = threadIdx.x; t < n; t += blockDim.x) vk[t] = cmul(ristar[t], f);
        for (int64_t t = threadIdx.x; t < m; t += blockDim.x) uk[t] = rjstar[t];
        __syncthreads();
        rank = (int)k + 1;
        // update_norm_estimate (aca.rs:224-241): the products with every
        // earlier rank one warp each, summed in rank order by one thread
        double nk = bnsq(uk, m, sh) * bnsq(vk, n, sh);
        {
            const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
            for (int t = warp; t < k; t += nw) {
                const double2* ut = U + (size_t)t * m;
                const double2* vt = V + (size_t)t * n;
                z2 du = make_double2(0, 0), dv = make_double2(0, 0);
                for (int64_t i = lane; i < m; i += 32) cfma(du, ut[i], uk[i]);
                for (int64_t j = lane; j < n; j += 32) cfma(dv, vt[j], vk[j]);
                du = wsum2(du);
                dv = wsum2(dv);
                if (lane == 0) s_prod[t] = 2.0 * hypot(du.x, du.y) * hypot(dv.x, dv.y);
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            double add = 0;
            for (int t = 0; t < k; ++t) add += s_prod[t];
            s_total += nk;
            s_total += add;
            double step = sqrt(nk) / sqrt(s_total);
            s_stop = step < tol / 50.0;
            s_istar = istar;
            s_jstar = jstar;
        }
        __syncthreads();
        if (s_stop) break;
        // reference row / column updates
        if (s_iref == istar) {
            if (threadIdx.x == 0) {
                int64_t v = s_iref;
                if (iex[v]) {
                    v = rng_uniform_incl(rng, (uint32_t)(nr - 1));
                    for (int64_t t = 0; t < nr - 1; ++t) {
                        v = (v + 1) % nr;
                        if (!iex[v]) break;
                    }
                }
                s_iref = v;
            }
            __syncthreads();
            aca_res_row(g, L, rows, cols, U, V, rank, s_iref, riref);
        } else {
            const z2 c = uk[s_iref];
            for (int64_t t = threadIdx.x; t < n; t += blockDim.x) cfma(riref[t], cneg(c), vk[t]);
            __syncthreads();
        }
        if (s_jref == jstar) {
            if (threadIdx.x == 0) {
                int64_t v = s_jref;
                if (jex[v]) {
                    v = rng_uniform_incl(rng, (uint32_t)(nr - 1));
                    for (int64_t t = 0; t < nr - 1; ++t) {
                        v = (v + 1) % nr;
                        if (!jex[v]) break;
                    }
                }
                s_jref = v;
            }
            __syncthreads();
            aca_res_col(g, L, rows, cols, U, V, rank, s_jref, rjref);
        } else {
            const z2 c = vk[s_jref];
            for (int64_t t = threadIdx.x; t < m; t += blockDim.x) cfma(rjref[t], cneg(c), uk[t]);
            __syncthreads();
        }
    }
    if (threadIdx.x == 0) {
        L.rank = rank;
        L.norm = sqrt(s_total);
    }
}

// ---------------------------------------------------------------------------
// QR + SVD recompression (aca.rs:137-179) and the ab-initio norm estimate
// (aca.rs:212-222).  Householder QR of U (m x r) and V (n x r) in place (the
// reflectors overwrite the factor, R goes to scratch), SVD of R_u R_v^T by
// one-sided Jacobi, truncation at s < tol * cumulative sum (+1, at least 1),
// then U <- Q_u W Sigma and V <- Q_v Z with Z = (V^H)^T (plain transpose, the
// factors pair as u v^T).
__device__ void house_qr_dev(double2* A, int64_t m, int r, double2* R, double2* tau, double* sh) {
    // A: m x r column-major; on exit the reflectors v_k (v_k[k] = 1 implied
    // by storing the full vector) are kept in A below and on the diagonal.
    // Column k's reflector comes from two block reductions; its application
    // to the later columns runs one warp per column (warp reductions, one
    // barrier per k).
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    __shared__ double2 s_alpha, s_tau;
    for (int k = 0; k < r; ++k) {
        double2* a = A + (size_t)k * m;
        double nx2 = 0;
        for (int64_t i = k + threadIdx.x; i < m; i += blockDim.x) nx2 += cnorm2(a[i]);
        double nx = sqrt(bsum(nx2, sh));
        if (threadIdx.x == 0) {
            z2 x0 = a[k];
            double ax0 = hypot(x0.x, x0.y);
            z2 ph = ax0 == 0 ? make_double2(1.0, 0.0) : make_double2(x0.x / ax0, x0.y / ax0);
            s_alpha = cscale(cneg(ph), nx);
        }
        __syncthreads();
        // v = x - alpha e_k (stored in a[k..m))
        if (threadIdx.x == 0) a[k] = csub(a[k], s_alpha);
        __syncthreads();
        double vn2 = 0;
        for (int64_t i = k + threadIdx.x; i < m; i += blockDim.x) vn2 += cnorm2(a[i]);
        vn2 = bsum(vn2, sh);
        if (threadIdx.x == 0) s_tau = make_double2(vn2 == 0 ? 0.0 : 2.0 / vn2, 0.0);
        __syncthreads();
        const double tk = s_tau.x;
        // apply H_k to columns j > k, one warp per column
        for (int j = k + 1 + warp; j < r; j += nw) {
            double2* c = A + (size_t)j * m;
            z2 d = make_double2(0, 0);
            for (int64_t i = k + lane; i < m; i += 32) cfma(d, cconj(a[i]), c[i]);
            d = cscale(wsum2(d), tk);
            for (int64_t i = k + lane; i < m; i += 32) cfma(c[i], cneg(a[i]), d);
        }
        if (threadIdx.x == 0) tau[k] = make_double2(tk, 0.0);
        for (int i = threadIdx.x; i < r; i += blockDim.x)
            R[(size_t)k * r + i] = i == k ? s_alpha : make_double2(0, 0);
        __syncthreads();
    }
    // R above the diagonal lives in rows < k of columns k (read after the loop)
    for (int j = 0; j < r; ++j)
        for (int i = threadIdx.x; i < j; i += blockDim.x) R[(size_t)j * r + i] = A[(size_t)j * m + i];
    __syncthreads();
}

// out (m x c) = Q [B; 0] where Q = H_0 ... H_{r-1} (reflectors in A), B r x c;
// one warp per output column for each reflector.
__device__ void house_apply_dev(const double2* A, int64_t m, int r, const double2* tau, const double2* B, int c,
                                double2* out, double* sh) {
    (void)sh;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int j = 0; j < c; ++j)
        for (int64_t i = threadIdx.x; i < m; i += blockDim.x)
            out[(size_t)j * m + i] = i < r ? B[(size_t)j * r + i] : make_double2(0, 0);
    __syncthreads();
    for (int k = r - 1; k >= 0; --k) {
        const double2* v = A + (size_t)k * m;
        const double tk = tau[k].x;
        if (tk == 0.0) continue;
        for (int j = warp; j < c; j += nw) {
            double2* o = out + (size_t)j * m;
            z2 d = make_double2(0, 0);
            for (int64_t i = k + lane; i < m; i += 32) cfma(d, cconj(v[i]), o[i]);
            d = cscale(wsum2(d), tk);
            for (int64_t i = k + lane; i < m; i += 32) cfma(o[i], cneg(v[i]), d);
        }
        __syncthreads();
    }
}

// One-sided Jacobi SVD of the r x r matrix M (overwritten): M = W S Vh with S
// descending.  Each sweep visits every column pair once in the round-robin
// order: r' - 1 steps (r' = r rounded up to even) of r' / 2 disjoint pairs,
// one warp per pair, one barrier per step.
__device__ void jacobi_svd_dev(double2* M, double2* Vm, int r, double* S, int* perm, double* sh) {
    (void)sh;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int j = 0; j < r; ++j)
        for (int i = threadIdx.x; i < r; i += blockDim.x) Vm[(size_t)j * r + i] = make_double2(i == j, 0.0);
    __syncthreads();
    __shared__ unsigned long long s_off;  // largest |cos angle| of a sweep, as the bits of a positive double
    const int rr = r + (r & 1);           // players of the round robin (index r: a bye when r is odd)
    for (int sweep = 0; sweep < 60; ++sweep) {
        if (threadIdx.x == 0) s_off = 0ull;
        __syncthreads();
        for (int step = 0; step < rr - 1; ++step) {
            for (int pi = warp; pi < rr / 2; pi += nw) {
                // circle method: player 0 fixed, the others rotate by `step`
                const int a0 = pi == 0 ? 0 : 1 + (pi - 1 + step) % (rr - 1);
                const int b0 = 1 + (rr - 2 - pi + step) % (rr - 1);
                const int p = min(a0, b0), q = max(a0, b0);
                if (q >= r) continue;  // the bye
                double2* up = M + (size_t)p * r;
                double2* uq = M + (size_t)q * r;
                double a = 0, b = 0;
                z2 cc = make_double2(0, 0);
                for (int i = lane; i < r; i += 32) {
                    a += cnorm2(up[i]);
                    b += cnorm2(uq[i]);
                    cfma(cc, cconj(up[i]), uq[i]);
                }
                a = wsum(a);
                b = wsum(b);
                cc = wsum2(cc);
                const double ac = hypot(cc.x, cc.y);
                if (ac == 0 || ac <= 1e-15 * sqrt(a * b)) continue;
                if (lane == 0) atomicMax(&s_off, (unsigned long long)__double_as_longlong(ac / sqrt(a * b)));
                const double zeta = (b - a) / (2.0 * ac);
                const double t = (zeta >= 0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
                const double cs = 1.0 / sqrt(1.0 + t * t), sn = cs * t;
                const z2 e = make_double2(cc.x / ac, cc.y / ac);
                const z2 se = cscale(e, sn), sce = cscale(cconj(e), sn);
                double2* vp = Vm + (size_t)p * r;
                double2* vq = Vm + (size_t)q * r;
                for (int i = lane; i < r; i += 32) {
                    z2 x = up[i], y = uq[i];
                    up[i] = csub(cscale(x, cs), cmul(sce, y));
                    uq[i] = cadd(cmul(se, x), cscale(y, cs));
                    z2 vx = vp[i], vy = vq[i];
                    vp[i] = csub(cscale(vx, cs), cmul(sce, vy));
                    vq[i] = cadd(cmul(se, vx), cscale(vy, cs));
                }
            }
            __syncthreads();
        }
        const double off = __longlong_as_double((long long)s_off);
        __syncthreads();
        if (off < 1e-15) break;
    }
    // singular values, descending order (stable)
    for (int j = warp; j < r; j += nw) {
        double v = 0;
        for (int i = lane; i < r; i += 32) v += cnorm2(M[(size_t)j * r + i]);
        v = wsum(v);
        if (lane == 0) S[j] = sqrt(v);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int j = 0; j < r; ++j) perm[j] = j;
        for (int a = 0; a < r; ++a)
            for (int b = a + 1; b < r; ++b)
                if (S[perm[b]] > S[perm[a]]) { int t = perm[a]; perm[a] = perm[b]; perm[b] = t; }
    }
    __syncthreads();
}

__global__ void __launch_bounds__(LEAF_THREADS) hm_recompress_kernel(HLeaf* __restrict__ leaves,
                                                                     const int32_t* __restrict__ list,
                                                                     double2* __restrict__ store,
                                                                     double2* __restrict__ scr,
                                                                     const int64_t* __restrict__ scr2_off,
                                                                     double tol) {
    __shared__ double sh[48];
    HLeaf& L = leaves[list[blockIdx.x]];
    const int r = L.rank;
    const int64_t m = L.m, n = L.n;
    double2* U = store + L.store_off;
    double2* V = U + (size_t)m * L.kmax;
    double2* w = scr + scr2_off[blockIdx.x];
    double2* Ru = w;
    double2* Rv = Ru + (size_t)r * r;
    double2* RR = Rv + (size_t)r * r;
    double2* Vm = RR + (size_t)r * r;
    double2* B = Vm + (size_t)r * r;
    double2* tauu = B + (size_t)r * r;
    double2* tauv = tauu + r;
    double2* outU = tauv + r;             // m x r
    double2* outV = outU + (size_t)m * r; // n x r
    double* S = reinterpret_cast<double*>(outV + (size_t)n * r);
    int* perm = reinterpret_cast<int*>(S + r);
    house_qr_dev(U, m, r, Ru, tauu, sh);
    house_qr_dev(V, n, r, Rv, tauv, sh);
    // RR = R_u R_v^T
    for (int t = threadIdx.x; t < r * r; t += blockDim.x) {
        int i = t % r, j = t / r;
        z2 acc = make_double2(0, 0);
        for (int l = 0; l < r; ++l) cfma(acc, Ru[(size_t)l * r + i], Rv[(size_t)l * r + j]);
        RR[(size_t)j * r + i] = acc;
    }
    __syncthreads();
    jacobi_svd_dev(RR, Vm, r, S, perm, sh);
    // truncation (aca.rs:162-171)
    __shared__ int s_keep;
    if (threadIdx.x == 0) {
        int index = 0;
        double sum = 0;
        for (int t = 0; t < r; ++t) {
            double sv = S[perm[t]];
            sum += sv;
            if (sv < tol * sum) break;
            index++;
        }
        index = index + 1 < r ? index + 1 : r;
        if (index < 1) index = 1;
        s_keep = index;
    }
    __syncthreads();
    const int keep = s_keep;
    // U_new = Q_u (W Sigma): W column t = RR column perm[t] / S (so W S = RR col)
    for (int t = 0; t < keep; ++t)
        for (int i = threadIdx.x; i < r; i += blockDim.x) B[(size_t)t * r + i] = RR[(size_t)perm[t] * r + i];
    __syncthreads();
    house_apply_dev(U, m, r, tauu, B, keep, outU, sh);
    // V_new = Q_v Z, Z column t = (Vh row t)^T = conj(Vm column perm[t])
    for (int t = 0; t < keep; ++t)
        for (int i = threadIdx.x; i < r; i += blockDim.x) B[(size_t)t * r + i] = cconj(Vm[(size_t)perm[t] * r + i]);
    __syncthreads();
    house_apply_dev(V, n, r, tauv, B, keep, outV, sh);
    for (int t = 0; t < keep; ++t) {
        for (int64_t i = threadIdx.x; i < m; i += blockDim.x) U[(size_t)t * m + i] = outU[(size_t)t * m + i];
        for (int64_t i = threadIdx.x; i < n; i += blockDim.x) V[(size_t)t * n + i] = outV[(size_t)t * n + i];
    }
    __syncthreads();
    // calculate_norm_estimate (aca.rs:212-222): for each rank a, its products
    // with the earlier ranks one warp each, summed in rank order by one thread
    __shared__ double s_prod[256];  // keep <= kmax <= 256
    double tot = 0;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int a = 0; a < keep; ++a) {
        double nu = bnsq(U + (size_t)a * m, m, sh), nv = bnsq(V + (size_t)a * n, n, sh);
        for (int b = warp; b < a; b += nw) {
            z2 du = make_double2(0, 0), dv = make_double2(0, 0);
            for (int64_t i = lane; i < m; i += 32) cfma(du, U[(size_t)a * m + i], U[(size_t)b * m + i]);
            for (int64_t j = lane; j < n; j += 32) cfma(dv, V[(size_t)a * n + j], V[(size_t)b * n + j]);
            du = wsum2(du);
            dv = wsum2(dv);
            if (lane == 0) s_prod[b] = 2.0 * hypot(du.x, du.y) * hypot(dv.x, dv.y);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            tot += nu * nv;
            for (int b = 0; b < a; ++b) tot += s_prod[b];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        L.rank = keep;
        L.norm = sqrt(tot);
    }
}

// Frobenius norm of dense leaves.
__global__ void hm_dense_norm_kernel(HLeaf* __restrict__ leaves, const int32_t* __restrict__ list,
                                     const double2* __restrict__ store) {
    __shared__ double sh[48];
    HLeaf& L = leaves[list[blockIdx.x]];
    double v = bnsq(store + L.store_off, L.m * L.n, sh);
    if (threadIdx.x == 0) L.norm = sqrt(v);
}

// ---------------------------------------------------------------------------
// Mat-vec: every leaf multiplies its gathered slice of x (alpha applied), the
// row reduction adds the slices of each global row in leaf order.
__global__ void __launch_bounds__(LEAF_THREADS) hm_leaf_mv_kernel(const HLeaf* __restrict__ leaves,
                                                                  const int64_t* __restrict__ rows,
                                                                  const int64_t* __restrict__ cols,
                                                                  const double2* __restrict__ store, GmBatch bt,
                                                                  int mode, const double2* __restrict__ xin,
                                                                  z2 alpha, double2* __restrict__ y) {
    __shared__ double sh[48];
    __shared__ double2 tks[64];
    const double2* x = xin;
    if (bt.st) {
        const GmState& st = bt.st[0];
        if (!gm_apply_active(bt, st, mode)) return;
        x = (mode == MV_Q) ? bt.Q + (size_t)st.k * bt.n : bt.X;
    }
    const HLeaf L = leaves[blockIdx.x];
    const double2* D = store + L.store_off;
    double2* yo = y + L.y_off;
    if (!L.adm) {
        for (int64_t i = threadIdx.x; i < L.m; i += blockDim.x) {
            z2 acc = make_double2(0, 0);
            for (int64_t j = 0; j < L.n; ++j) cfma(acc, D[(size_t)j * L.m + i], x[cols[L.col_off + j]]);
            yo[i] = cmul(alpha, acc);
        }
        return;
    }
    const double2* U = D;
    const double2* V = U + (size_t)L.m * L.kmax;
    for (int i = threadIdx.x; i < L.m; i += blockDim.x) yo[i] = make_double2(0, 0);
    for (int k0 = 0; k0 < L.rank; k0 += 64) {
        const int kc = min(64, L.rank - k0);
        for (int k = 0; k < kc; ++k) {
            const double2* vk = V + (size_t)(k0 + k) * L.n;
            z2 acc = make_double2(0, 0);
            for (int64_t j = threadIdx.x; j < L.n; j += blockDim.x) cfma(acc, vk[j], x[cols[L.col_off + j]]);
            acc = bsum2(acc, sh);
            if (threadIdx.x == 0) tks[k] = cmul(alpha, acc);  // alpha * (v_k . x), aca.rs:187-193
        }
        __syncthreads();
        for (int64_t i = threadIdx.x; i < L.m; i += blockDim.x) {
            z2 a = yo[i];
            for (int k = 0; k < kc; ++k) cfma(a, U[(size_t)(k0 + k) * L.m + i], tks[k]);
            yo[i] = a;
        }
        __syncthreads();
    }
}

// out[i] = beta * out[i] + sum over the leaves covering row i (fixed order).
__global__ void hm_row_reduce_kernel(int64_t n, const int64_t* __restrict__ rowptr, const int64_t* __restrict__ ent,
                                     const double2* __restrict__ y, GmBatch bt, int mode, z2 beta,
                                     double2* __restrict__ out) {
    if (bt.st) {
        const GmState& st = bt.st[0];
        if (!gm_apply_active(bt, st, mode)) return;
    }
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    z2 acc = (beta.x == 0.0 && beta.y == 0.0) ? make_double2(0, 0) : cmul(beta, out[i]);
    for (int64_t t = rowptr[i]; t < rowptr[i + 1]; ++t) acc = cadd(acc, y[ent[t]]);
    out[i] = acc;
}

// ---------------------------------------------------------------------------
static GenParams gen_params(const Problem& p, int side) {
    GenParams g;
    g.kp = kparams(p);
    cd a, b;
    if (side) lhs_factors(p, a, b); else rhs_factors(p, a, b);
    g.alpha = make_double2(a.re, a.im);
    g.beta = make_double2(b.re, b.im);
    g.npad = p.geo.npad;
    g.geo = p.geo.arr(0);
    return g;
}

constexpr int ACA_RMAX = 256;  // also the size of the ACA kernel's s_prod

// The cluster tree and block leaves of a problem's collocation points (they
// depend on the geometry, the leaf size and eta only, not on the frequency),
// built on the device.
struct HTrees {
    std::shared_ptr<Forest> F;
    std::vector<BlockLeaf> bl;
};

static std::shared_ptr<HTrees> build_trees(Context& c, const Problem& p) {
    auto T = std::make_shared<HTrees>();
    T->F = build_forest(c, std::vector<const Problem*>{&p}, p.in.hm_leaf);
    T->bl = forest_block_leaves(c, *T->F, p.in.hm_eta);
    return T;
}

// trees: the problem's trees from an earlier build (several frequencies of
// one body), or null to build them here.
std::unique_ptr<HMatrixDev> hmatrix_build(Context& c, const Problem& p, int side,
                                          std::shared_ptr<HTrees> trees = nullptr) {
    auto H = std::make_unique<HMatrixDev>();
    const int64_t n = p.n;
    H->n = n;
    if (!trees) trees = build_trees(c, p);
    const Forest& F = *trees->F;
    // every cluster is a range of the cluster-order permutation, so the row
    // and column lists of all leaves are that one array
    H->rows = F.perm;
    H->cols = F.perm;
    int64_t store = 0, scratch = 0, yoff = 0;
    for (const BlockLeaf& t : trees->bl) {
        const TreeNode& r = F.nodes[(size_t)t.r];
        const TreeNode& cc = F.nodes[(size_t)t.c];
        HLeaf L{};
        L.row_off = r.begin;
        L.m = r.end - r.begin;
        L.col_off = cc.begin;
        L.n = cc.end - cc.begin;
        L.adm = t.adm;
        L.store_off = store;
        L.y_off = yoff;
        yoff += L.m;
        if (L.adm) {
            L.kmax = (int32_t)std::min<int64_t>(std::min(L.m, L.n), ACA_RMAX);
            store += (L.m + L.n) * L.kmax;
            L.scratch_off = scratch;
            scratch += 2 * (L.m + L.n) + (L.m + L.n + 15) / 16 + 2;
        } else {
            L.kmax = 0;
            store += L.m * L.n;
        }
        H->leaves.push_back(L);
    }
    // device copies
    const size_t nl = H->leaves.size();
    H->d_leaves.ensure(sizeof(HLeaf) * nl);
    H->d_rows.ensure(sizeof(int64_t) * std::max<size_t>(H->rows.size(), 1));
    H->d_cols.ensure(sizeof(int64_t) * std::max<size_t>(H->cols.size(), 1));
    H->d_store.ensure(sizeof(double2) * (size_t)std::max<int64_t>(store, 1));
    H->d_scratch.ensure(sizeof(double2) * (size_t)std::max<int64_t>(scratch, 1));
    H->d_y.ensure(sizeof(double2) * (size_t)std::max<int64_t>(yoff, 1));
    BEM_CUDA(cudaMemcpyAsync(H->d_leaves.p, H->leaves.data(), sizeof(HLeaf) * nl, cudaMemcpyHostToDevice, c.stream));
    BEM_CUDA(cudaMemcpyAsync(H->d_rows.p, F.d_perm.p, sizeof(int64_t) * H->rows.size(), cudaMemcpyDeviceToDevice,
                             c.stream));
    BEM_CUDA(cudaMemcpyAsync(H->d_cols.p, F.d_perm.p, sizeof(int64_t) * H->cols.size(), cudaMemcpyDeviceToDevice,
                             c.stream));
    std::vector<int32_t> adm_list, dense_list;
    for (size_t b = 0; b < nl; ++b) (H->leaves[b].adm ? adm_list : dense_list).push_back((int32_t)b);
    DevBuf d_adm, d_dense;
    d_adm.ensure(sizeof(int32_t) * std::max<size_t>(adm_list.size(), 1));
    d_dense.ensure(sizeof(int32_t) * std::max<size_t>(dense_list.size(), 1));
    BEM_CUDA(cudaMemcpyAsync(d_adm.p, adm_list.data(), sizeof(int32_t) * adm_list.size(), cudaMemcpyHostToDevice,
                             c.stream));
    BEM_CUDA(cudaMemcpyAsync(d_dense.p, dense_list.data(), sizeof(int32_t) * dense_list.size(),
                             cudaMemcpyHostToDevice, c.stream));
    GenParams g = gen_params(p, side);
    HLeaf* dl = H->d_leaves.as<HLeaf>();
    if (!dense_list.empty()) {
        hm_dense_fill_kernel<<<(unsigned)dense_list.size(), LEAF_THREADS, 0, c.stream>>>(
            dl, d_dense.as<int32_t>(), H->d_rows.as<int64_t>(), H->d_cols.as<int64_t>(), g, H->d_store.as<double2>());
        BEM_CHECK_LAUNCH(&c);
        hm_dense_norm_kernel<<<(unsigned)dense_list.size(), LEAF_THREADS, 0, c.stream>>>(dl, d_dense.as<int32_t>(),
                                                                                         H->d_store.as<double2>());
        BEM_CHECK_LAUNCH(&c);
    }
    if (!adm_list.empty()) {
        int* err = device_err(c);
        BEM_CUDA(cudaMemsetAsync(err, 0, sizeof(int), c.stream));
        hm_aca_kernel<<<(unsigned)adm_list.size(), LEAF_THREADS, 0, c.stream>>>(
            dl, d_adm.as<int32_t>(), H->d_rows.as<int64_t>(), H->d_cols.as<int64_t>(), g, H->d_store.as<double2>(),
            H->d_scratch.as<double2>(), p.in.hm_aca_tol, err);
        BEM_CHECK_LAUNCH(&c);
        int herr = 0;
        BEM_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
        BEM_CUDA(cudaMemcpyAsync(H->leaves.data(), dl, sizeof(HLeaf) * nl, cudaMemcpyDeviceToHost, c.stream));
        c.sync();
        require(herr == 0, "ACA rank exceeded the storage cap of " + std::to_string(ACA_RMAX),
                BEM_ERR_NOT_CONVERGED);
        // recompression scratch sized by the ranks just found
        std::vector<int64_t> off(adm_list.size());
        int64_t tot = 0;
        for (size_t a = 0; a < adm_list.size(); ++a) {
            const HLeaf& L = H->leaves[(size_t)adm_list[a]];
            int64_t r = L.rank;
            off[a] = tot;
            tot += 5 * r * r + 2 * r + (L.m + L.n) * r + r + r / 2 + 2;
        }
        DevBuf d_off, d_scr2;
        d_off.ensure(sizeof(int64_t) * off.size());
        d_scr2.ensure(sizeof(double2) * (size_t)std::max<int64_t>(tot, 1));
        BEM_CUDA(cudaMemcpyAsync(d_off.p, off.data(), sizeof(int64_t) * off.size(), cudaMemcpyHostToDevice, c.stream));
        hm_recompress_kernel<<<(unsigned)adm_list.size(), LEAF_THREADS, 0, c.stream>>>(
            dl, d_adm.as<int32_t>(), H->d_store.as<double2>(), d_scr2.as<double2>(), d_off.as<int64_t>(),
            p.in.hm_aca_tol);
        BEM_CHECK_LAUNCH(&c);
        c.sync();
    }
    BEM_CUDA(cudaMemcpyAsync(H->leaves.data(), dl, sizeof(HLeaf) * nl, cudaMemcpyDeviceToHost, c.stream));
    c.sync();
    // update_norm (h_matrix.rs:189-196): dense leaves first, then low-rank
    double nrm = 0;
    for (auto& L : H->leaves)
        if (!L.adm) nrm += L.norm;
    for (auto& L : H->leaves)
        if (L.adm) nrm += L.norm;
    H->norm = nrm;
    for (auto& L : H->leaves) {
        if (L.adm) {
            H->nadm++;
            H->stored += L.rank * (L.m + L.n);
            H->rank_sum += L.rank;
        } else {
            H->ninadm++;
            H->stored += L.m * L.n;
        }
    }
    // row CSR over the leaves' output slices (leaf order)
    std::vector<int64_t> cnt((size_t)n + 1, 0);
    for (auto& L : H->leaves)
        for (int64_t i = 0; i < L.m; ++i) cnt[(size_t)H->rows[(size_t)(L.row_off + i)] + 1]++;
    for (int64_t i = 0; i < n; ++i) cnt[(size_t)i + 1] += cnt[(size_t)i];
    std::vector<int64_t> ent((size_t)cnt[(size_t)n]), pos(cnt.begin(), cnt.end() - 1);
    for (auto& L : H->leaves)
        for (int64_t i = 0; i < L.m; ++i) ent[(size_t)pos[(size_t)H->rows[(size_t)(L.row_off + i)]]++] = L.y_off + i;
    H->d_rowptr.ensure(sizeof(int64_t) * cnt.size());
    H->d_rowent.ensure(sizeof(int64_t) * std::max<size_t>(ent.size(), 1));
    BEM_CUDA(cudaMemcpyAsync(H->d_rowptr.p, cnt.data(), sizeof(int64_t) * cnt.size(), cudaMemcpyHostToDevice,
                             c.stream));
    BEM_CUDA(cudaMemcpyAsync(H->d_rowent.p, ent.data(), sizeof(int64_t) * ent.size(), cudaMemcpyHostToDevice,
                             c.stream));
    BEM_CUDA(cudaMemcpyAsync(H->d_leaves.p, H->leaves.data(), sizeof(HLeaf) * nl, cudaMemcpyHostToDevice, c.stream));
    c.sync();
    return H;
}

void hmatrix_gemv(Context& c, const HMatrixDev& H, cd alpha, const double2* x, cd beta, double2* b);

// The built leaves for the mixed form's repacking (hmixed.cu): index lists,
// ranks, norms and the device data of the FP64 build, kept alive by `keep`.
HBuilt hmatrix_build_view(Context& c, const Problem& p, int side, std::shared_ptr<void>* tree_cache) {
    std::shared_ptr<HTrees> trees;
    if (tree_cache && *tree_cache) trees = std::static_pointer_cast<HTrees>(*tree_cache);
    if (!trees) {
        trees = build_trees(c, p);
        if (tree_cache) *tree_cache = trees;
    }
    std::shared_ptr<HMatrixDev> H(hmatrix_build(c, p, side, trees).release());
    HBuilt v;
    v.n = H->n;
    v.norm = H->norm;
    v.leaves.reserve(H->leaves.size());
    for (const HLeaf& L : H->leaves)
        v.leaves.push_back(HLeafView{L.row_off, L.m, L.col_off, L.n, L.store_off, L.adm, L.kmax, L.rank, L.norm});
    v.rows = H->rows;
    v.cols = H->cols;
    v.d_rows = H->d_rows.as<int64_t>();
    v.d_cols = H->d_cols.as<int64_t>();
    v.d_store = H->d_store.as<double2>();
    v.keep = H;
    return v;
}

std::shared_ptr<const Forest> hmatrix_forest(Context& c, const Problem& p, std::shared_ptr<void>* tree_cache) {
    std::shared_ptr<HTrees> trees;
    if (tree_cache && *tree_cache) trees = std::static_pointer_cast<HTrees>(*tree_cache);
    if (!trees) {
        trees = build_trees(c, p);
        if (tree_cache) *tree_cache = trees;
    }
    return trees->F;
}

// out = (alpha H + beta G) 1 with the FP64 H-matrix of `side`
// (h_matrix.rs:218-234 applied to the constant vector), device memory.
void hmatrix_row_sums(Context& c, const Problem& p, int side, double2* out) {
    auto H = hmatrix_build(c, p, side);
    DevBuf ones;
    ones.ensure(sizeof(double2) * (size_t)p.n);
    std::vector<double2> h((size_t)p.n, make_double2(1.0, 0.0));
    BEM_CUDA(cudaMemcpyAsync(ones.p, h.data(), sizeof(double2) * (size_t)p.n, cudaMemcpyHostToDevice, c.stream));
    hmatrix_gemv(c, *H, {1.0, 0.0}, ones.as<double2>(), {0.0, 0.0}, out);
    c.sync();
}

// b = alpha H x + beta b on device vectors (h_matrix.rs:218-234).
void hmatrix_gemv(Context& c, const HMatrixDev& H, cd alpha, const double2* x, cd beta, double2* b) {
    GmBatch none{};
    if (!H.leaves.empty()) {
        hm_leaf_mv_kernel<<<(unsigned)H.leaves.size(), LEAF_THREADS, 0, c.stream>>>(
            H.d_leaves.as<HLeaf>(), H.d_rows.as<int64_t>(), H.d_cols.as<int64_t>(), H.d_store.as<double2>(), none, 0,
            x, make_double2(alpha.re, alpha.im), const_cast<double2*>(H.d_y.as<double2>()));
        BEM_CHECK_LAUNCH(&c);
    }
    hm_row_reduce_kernel<<<(unsigned)((H.n + 255) / 256), 256, 0, c.stream>>>(
        H.n, H.d_rowptr.as<int64_t>(), H.d_rowent.as<int64_t>(), H.d_y.as<double2>(), none, 0,
        make_double2(beta.re, beta.im), b);
    BEM_CHECK_LAUNCH(&c);
}

// GMRES operator hook: W = H v, predicated on the (single) system's state.
static void hm_apply_hook(Context& c, GmWorkspace& ws, int mode, void* user) {
    const HMatrixDev& H = *static_cast<const HMatrixDev*>(user);
    hm_leaf_mv_kernel<<<(unsigned)H.leaves.size(), LEAF_THREADS, 0, c.stream>>>(
        H.d_leaves.as<HLeaf>(), H.d_rows.as<int64_t>(), H.d_cols.as<int64_t>(), H.d_store.as<double2>(), ws.bt, mode,
        nullptr, make_double2(1.0, 0.0), const_cast<double2*>(H.d_y.as<double2>()));
    BEM_CHECK_LAUNCH(&c);
    hm_row_reduce_kernel<<<(unsigned)((H.n + 255) / 256), 256, 0, c.stream>>>(
        H.n, H.d_rowptr.as<int64_t>(), H.d_rowent.as<int64_t>(), H.d_y.as<double2>(), ws.bt, mode,
        make_double2(0.0, 0.0), ws.bt.W);
    BEM_CHECK_LAUNCH(&c);
}

GmresResult gmres_hmatrix(Context& c, const HMatrixDev& H, int64_t max_it, double tol, double2* x) {
    const int64_t n = H.n;
    if (max_it <= 0) max_it = 1000;
    if (max_it > n) max_it = n;
    if (tol <= 0.0) tol = 1e-5;
    int m = (int)std::ceil(std::sqrt((double)max_it));
    int64_t restarts = max_it / m;
    GmWorkspace ws;
    gm_prepare(c, ws, 1, n, m, nullptr, n, 0, false, true);
    ws.hook = hm_apply_hook;
    ws.hook_user = const_cast<HMatrixDev*>(&H);
    BEM_CUDA(cudaMemcpyAsync(ws.bt.B, x, sizeof(double2) * n, cudaMemcpyDeviceToDevice, c.stream));
    BEM_CUDA(cudaMemcpyAsync(ws.anorm, &H.norm, sizeof(double), cudaMemcpyHostToDevice, c.stream));
    gm_init(c, ws, tol, restarts);
    gm_run(c, ws, 0, restarts * (int64_t)m + 1);
    std::vector<GmState> st;
    gm_read_states(c, ws, st);
    BEM_CUDA(cudaMemcpyAsync(x, ws.bt.X, sizeof(double2) * n, cudaMemcpyDeviceToDevice, c.stream));
    c.sync();
    GmresResult r;
    r.num_mv = st[0].num_mv;
    r.restarts = st[0].restarts + (st[0].converged ? 1 : 0);
    r.iterations = st[0].iterations;
    r.error = st[0].error;
    r.flag = st[0].converged ? 1 : 2;
    return r;
}

// solve.rs:74-150 get_surface_hmatrix.
void solve_surface_hmatrix(Context& c, const Problem& p, const double2* d_rhs_inc, double2* d_phi, double2* d_vn,
                           bem_solve_report* rep) {
    const int64_t n = p.n;
    DevBuf vb;
    vb.ensure(sizeof(double2) * 2 * n);
    double2* rhs = vb.as<double2>();
    double2* fillv = rhs + n;
    BEM_CUDA(cudaMemcpyAsync(rhs, d_rhs_inc, sizeof(double2) * n, cudaMemcpyDeviceToDevice, c.stream));
    const bool zero_bc = p.in.bc_value[0] == 0.0 && p.in.bc_value[1] == 0.0;
    cd bcv = {p.in.bc_value[0], p.in.bc_value[1]};
    if (p.in.bc_type == 2) {
        // rhs = 0 * rhs_inc + (-1) rhs
        launch_rhs_combine(c, n, -1.0, d_rhs_inc, {0, 0}, nullptr, rhs);
    } else {
        cd beta = p.in.bc_type == 0 ? cd{1.0, 0.0} : cd{-1.0, 0.0};
        if (!zero_bc) {
            auto Hr = hmatrix_build(c, p, 0);
            std::vector<double2> hv((size_t)n, make_double2(bcv.re, bcv.im));
            BEM_CUDA(cudaMemcpyAsync(fillv, hv.data(), sizeof(double2) * n, cudaMemcpyHostToDevice, c.stream));
            hmatrix_gemv(c, *Hr, {1.0, 0.0}, fillv, beta, rhs);
            c.sync();
        } else if (beta.re != 1.0) {
            launch_rhs_combine(c, n, -1.0, d_rhs_inc, {0, 0}, nullptr, rhs);
        }
    }
    auto Hl = hmatrix_build(c, p, 1);
    GmresResult r = gmres_hmatrix(c, *Hl, p.in.max_iterations, p.in.tolerance, rhs);
    if (rep) {
        rep->num_mv = r.num_mv;
        rep->restarts = r.restarts;
        rep->iterations = r.iterations;
        rep->backward_error = r.error;
        rep->flag = r.flag;
    }
    unpack_solution(c, p, rhs, d_phi, d_vn);
    c.sync();
}

}  // namespace bem

using namespace bem;

extern "C" {

BEM_API bem_status bem_hmatrix_build(bem_ctx* ctx, const bem_problem* pp, bem_side side, bem_hmatrix** out) {
    if (!ctx || !pp || !out) return BEM_ERR_BAD_INPUT;
    *out = nullptr;
    try {
        Context& c = ctx->c;
        BEM_CUDA(cudaSetDevice(c.device));
        auto H = hmatrix_build(c, pp->p, side == BEM_SIDE_LHS ? 1 : 0);
        *out = new bem_hmatrix{H.release(), ctx};
        return BEM_OK;
    } catch (const Error& e) {
        ctx->c.last_error = e.what();
        return e.status;
    } catch (const std::exception& e) {
        ctx->c.last_error = e.what();
        return BEM_ERR_CUDA;
    }
}

BEM_API void bem_hmatrix_destroy(bem_hmatrix* h) {
    if (!h) return;
    delete h->h;
    delete h;
}

BEM_API bem_status bem_hmatrix_gemv(bem_ctx* ctx, const bem_hmatrix* h, bem_cplx alpha, const bem_cplx* x,
                                    bem_cplx beta, bem_cplx* b) {
    if (!ctx || !h || !x || !b) return BEM_ERR_BAD_INPUT;
    try {
        Context& c = ctx->c;
        BEM_CUDA(cudaSetDevice(c.device));
        const int64_t n = h->h->n;
        DevBuf d;
        d.ensure(sizeof(double2) * 2 * n);
        double2* dx = d.as<double2>();
        double2* db = dx + n;
        BEM_CUDA(cudaMemcpyAsync(dx, x, sizeof(double2) * n, cudaMemcpyHostToDevice, c.stream));
        BEM_CUDA(cudaMemcpyAsync(db, b, sizeof(double2) * n, cudaMemcpyHostToDevice, c.stream));
        hmatrix_gemv(c, *h->h, {alpha.re, alpha.im}, dx, {beta.re, beta.im}, db);
        BEM_CUDA(cudaMemcpyAsync(b, db, sizeof(double2) * n, cudaMemcpyDeviceToHost, c.stream));
        c.sync();
        return BEM_OK;
    } catch (const Error& e) {
        ctx->c.last_error = e.what();
        return e.status;
    }
}

BEM_API double bem_hmatrix_norm(const bem_hmatrix* h) { return h ? h->h->norm : 0.0; }

BEM_API bem_status bem_hmatrix_stats(const bem_hmatrix* h, int64_t* s) {
    if (!h || !s) return BEM_ERR_BAD_INPUT;
    s[0] = h->h->nadm;
    s[1] = h->h->ninadm;
    s[2] = h->h->stored;
    s[3] = h->h->rank_sum;
    return BEM_OK;
}

BEM_API bem_status bem_hmatrix_to_full(bem_ctx* ctx, const bem_hmatrix* h, bem_cplx* A, int64_t lda) {
    if (!ctx || !h || !A || lda < h->h->n) return BEM_ERR_BAD_INPUT;
    // columns of the identity through the mat-vec kernels (h_matrix.rs:236-246)
    const int64_t n = h->h->n;
    std::vector<double2> e((size_t)n), col((size_t)n);
    try {
        Context& c = ctx->c;
        BEM_CUDA(cudaSetDevice(c.device));
        DevBuf d;
        d.ensure(sizeof(double2) * 2 * n);
        double2* dx = d.as<double2>();
        double2* db = dx + n;
        BEM_CUDA(cudaMemsetAsync(dx, 0, sizeof(double2) * n, c.stream));
        const double2 one = make_double2(1, 0), zero = make_double2(0, 0);
        for (int64_t j = 0; j < n; ++j) {
            if (j > 0) BEM_CUDA(cudaMemcpyAsync(dx + j - 1, &zero, sizeof(double2), cudaMemcpyHostToDevice, c.stream));
            BEM_CUDA(cudaMemcpyAsync(dx + j, &one, sizeof(double2), cudaMemcpyHostToDevice, c.stream));
            hmatrix_gemv(c, *h->h, {1.0, 0.0}, dx, {0.0, 0.0}, db);
            BEM_CUDA(cudaMemcpyAsync(A + j * lda, db, sizeof(double2) * n, cudaMemcpyDeviceToHost, c.stream));
            c.sync();
        }
        return BEM_OK;
    } catch (const Error& e) {
        ctx->c.last_error = e.what();
        return e.status;
    }
}

}  // extern "C"
