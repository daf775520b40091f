/*
 * bem_oracle.c -- CPU FP64 restatement of the cc_abstemious BEM hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle).  See bem_oracle.h for the scope and
 * the golden values that pin it.  Built with -ffp-contract=off and
 * -fcx-limited-range so that complex arithmetic follows num-complex 0.4.6's
 * textbook formulas and no fused multiply-adds are introduced.
 */
#include "bem_oracle.h"

#include <complex.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex cplx;
#define CPLX(p, i) ((p)[2 * (i)] + I * (p)[2 * (i) + 1])
static inline void cput(double* p, int64_t i, cplx v) { p[2 * i] = creal(v); p[2 * i + 1] = cimag(v); }
static const double PI = 3.14159265358979323846;

/* ======================================================================= */
/* rand 0.9.0 StdRng = rand_chacha 0.9 ChaCha12Rng, seeded by rand_core 0.9.3
 * SeedableRng::seed_from_u64 (PCG32 fill of the 32-byte key).  Used by
 * solve.rs:194-209 (test matrices) and aca.rs:64-68 (random reference pivots).
 * Output: 4 ChaCha blocks per refill (64-bit block counter in words 12-13,
 * stream 0 in words 14-15), consumed word by word (rand_core BlockRng). */
static inline uint32_t rotl32(uint32_t v, int c) { return (v << c) | (v >> (32 - c)); }
#define QR(a, b, c, d) \
    s[a] += s[b]; s[d] = rotl32(s[d] ^ s[a], 16); \
    s[c] += s[d]; s[b] = rotl32(s[b] ^ s[c], 12); \
    s[a] += s[b]; s[d] = rotl32(s[d] ^ s[a], 8);  \
    s[c] += s[d]; s[b] = rotl32(s[b] ^ s[c], 7);

static void chacha12_block(const uint32_t key[8], uint64_t ctr, uint32_t out[16]) {
    uint32_t st[16] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u,
                       key[0], key[1], key[2], key[3], key[4], key[5], key[6], key[7],
                       (uint32_t)ctr, (uint32_t)(ctr >> 32), 0u, 0u};
    uint32_t s[16];
    memcpy(s, st, sizeof s);
    for (int r = 0; r < 6; ++r) {
        QR(0, 4, 8, 12) QR(1, 5, 9, 13) QR(2, 6, 10, 14) QR(3, 7, 11, 15)
        QR(0, 5, 10, 15) QR(1, 6, 11, 12) QR(2, 7, 8, 13) QR(3, 4, 9, 14)
    }
    for (int i = 0; i < 16; ++i) out[i] = s[i] + st[i];
}

void oc_stdrng_seed(oc_stdrng* r, uint64_t state) {
    for (int i = 0; i < 8; ++i) {
        state = state * 6364136223846793005ull + 11634580027462260723ull;
        uint32_t xs = (uint32_t)(((state >> 18) ^ state) >> 27);
        uint32_t rot = (uint32_t)(state >> 59);
        r->key[i] = (xs >> rot) | (xs << ((32 - rot) & 31));
    }
    r->counter = 0;
    r->idx = 64;
}

static void stdrng_refill(oc_stdrng* r) {
    for (int b = 0; b < 4; ++b) chacha12_block(r->key, r->counter + (uint64_t)b, r->buf + 16 * b);
    r->counter += 4;
}

uint32_t oc_stdrng_u32(oc_stdrng* r) {
    if (r->idx >= 64) { stdrng_refill(r); r->idx = 0; }
    return r->buf[r->idx++];
}

uint64_t oc_stdrng_u64(oc_stdrng* r) {
    if (r->idx < 63) {
        uint64_t v = (uint64_t)r->buf[r->idx] | ((uint64_t)r->buf[r->idx + 1] << 32);
        r->idx += 2;
        return v;
    }
    if (r->idx >= 64) {
        stdrng_refill(r);
        r->idx = 2;
        return (uint64_t)r->buf[0] | ((uint64_t)r->buf[1] << 32);
    }
    uint64_t x = r->buf[63];
    stdrng_refill(r);
    r->idx = 1;
    return x | ((uint64_t)r->buf[0] << 32);
}

/* rand 0.9 StandardUniform for f64: 53 high bits times 2^-53. */
double oc_stdrng_f64(oc_stdrng* r) { return (double)(oc_stdrng_u64(r) >> 11) * (1.0 / 9007199254740992.0); }

/* rand 0.9 UniformUsize (ranges that fit in u32 sample 32-bit words): widening
   multiply with the rejection threshold (2^32 - range) mod range. */
uint64_t oc_uniform_usize_incl(oc_stdrng* r, uint64_t lo, uint64_t hi) {
    if (hi <= 0xffffffffull) {
        uint32_t range = (uint32_t)hi - (uint32_t)lo + 1u;
        if (range == 0) return lo + oc_stdrng_u32(r);
        uint32_t thresh = (uint32_t)(0u - range) % range;
        for (;;) {
            uint64_t m = (uint64_t)oc_stdrng_u32(r) * range;
            if ((uint32_t)m >= thresh) return lo + (m >> 32);
        }
    }
    uint64_t range = hi - lo + 1;
    uint64_t thresh = (0ull - range) % range;
    for (;;) {
        unsigned __int128 m = (unsigned __int128)oc_stdrng_u64(r) * range;
        if ((uint64_t)m >= thresh) return lo + (uint64_t)(m >> 64);
    }
}

/* solve.rs:194-209: A = n*I (on the leading diagonal) + U[0,1) re/im in
   column-major order, then b re/im. */
void oc_generate_random_ab(int64_t m, int64_t n, uint64_t seed, double* A, double* b) {
    oc_stdrng r;
    oc_stdrng_seed(&r, seed);
    memset(A, 0, sizeof(double) * 2 * m * n);
    for (int64_t i = 0; i < (m < n ? m : n); ++i) A[2 * (i * m + i)] = (double)n;
    for (int64_t j = 0; j < n; ++j)
        for (int64_t i = 0; i < m; ++i) {
            A[2 * (j * m + i)] += oc_stdrng_f64(&r);
            A[2 * (j * m + i) + 1] += oc_stdrng_f64(&r);
        }
    for (int64_t i = 0; i < n; ++i) {
        b[2 * i] = oc_stdrng_f64(&r);
        b[2 * i + 1] = oc_stdrng_f64(&r);
    }
}

/* ======================================================================= */
/* VTK legacy ASCII reader, reference dialect (mesh_data.rs:96-175): the first
 * integer of each CELLS row is the body id; bodies are created in the order
 * their ids first exceed the current body count. */
static char* read_file(const char* path, size_t* len) {
    FILE* f = fopen(path, "rb");
    if (!f) return NULL;
    fseek(f, 0, SEEK_END);
    long sz = ftell(f);
    fseek(f, 0, SEEK_SET);
    char* buf = (char*)malloc((size_t)sz + 1);
    if (!buf) { fclose(f); return NULL; }
    size_t got = fread(buf, 1, (size_t)sz, f);
    fclose(f);
    buf[got] = 0;
    *len = got;
    return buf;
}

static char* next_line(char** cur) {
    char* s = *cur;
    if (!s || !*s) return NULL;
    char* e = strchr(s, '\n');
    if (e) { *e = 0; *cur = e + 1; } else { *cur = s + strlen(s); }
    return s;
}

int oc_read_vtk(const char* path, oc_mesh* m) {
    memset(m, 0, sizeof *m);
    size_t len;
    char* buf = read_file(path, &len);
    if (!buf) { m->status = 1; return 1; }
    char* cur = buf;
    char* line;
    int64_t cap_conn = 0, nconn = 0;
    while ((line = next_line(&cur))) {
        char word[64];
        if (sscanf(line, " %63s", word) != 1) continue;
        if (!strcmp(word, "POINTS")) {
            long long np;
            if (sscanf(line, " %*s %lld", &np) != 1 || np < 0) { m->status = 2; break; }
            m->nnodes = np;
            m->nodes = (double*)malloc(sizeof(double) * 3 * (size_t)(np ? np : 1));
            for (int64_t i = 0; i < np; ++i) {
                char* l = next_line(&cur);
                if (!l || sscanf(l, "%lf %lf %lf", &m->nodes[3 * i], &m->nodes[3 * i + 1],
                                 &m->nodes[3 * i + 2]) != 3) { m->status = 3; goto done; }
            }
        } else if (!strcmp(word, "CELLS")) {
            long long ne;
            if (sscanf(line, " %*s %lld", &ne) != 1 || ne < 0) { m->status = 4; break; }
            m->nelem = ne;
            m->body = (int64_t*)calloc((size_t)(ne ? ne : 1), sizeof(int64_t));
            m->etype = (int32_t*)calloc((size_t)(ne ? ne : 1), sizeof(int32_t));
            m->conn_off = (int64_t*)calloc((size_t)ne + 1, sizeof(int64_t));
            cap_conn = 4 * ne + 16;
            m->conn = (int64_t*)malloc(sizeof(int64_t) * (size_t)cap_conn);
            for (int64_t i = 0; i < ne; ++i) {
                char* l = next_line(&cur);
                if (!l) { m->status = 5; goto done; }
                char* p = l;
                char* endp;
                long long v = strtoll(p, &endp, 10);
                if (endp == p) { m->status = 5; goto done; }
                m->body[i] = v;
                p = endp;
                for (;;) {
                    v = strtoll(p, &endp, 10);
                    if (endp == p) break;
                    if (nconn == cap_conn) {
                        cap_conn *= 2;
                        m->conn = (int64_t*)realloc(m->conn, sizeof(int64_t) * (size_t)cap_conn);
                    }
                    m->conn[nconn++] = v;
                    p = endp;
                }
                m->conn_off[i + 1] = nconn;
            }
        } else if (!strcmp(word, "CELL_TYPES")) {
            long long ne;
            if (sscanf(line, " %*s %lld", &ne) != 1 || ne < 0 || ne > m->nelem) { m->status = 6; break; }
            for (int64_t i = 0; i < ne; ++i) {
                char* l = next_line(&cur);
                int t;
                if (!l || sscanf(l, "%d", &t) != 1) { m->status = 7; goto done; }
                m->etype[i] = t;
            }
        }
    }
    /* bodies: mesh_data.rs:163-171 */
    for (int64_t e = 0; e < m->nelem; ++e) {
        if (m->body[e] < 1) { m->status = 8; break; }
        if (m->body[e] > m->nbodies) {
            if (m->body[e] != m->nbodies + 1) { m->status = 9; break; }
            m->nbodies++;
        }
    }
done:
    free(buf);
    return m->status;
}

void oc_mesh_free(oc_mesh* m) {
    free(m->nodes); free(m->body); free(m->etype); free(m->conn_off); free(m->conn);
    memset(m, 0, sizeof *m);
}

static inline double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static inline double norm3(const double* a) { return sqrt(dot3(a, a)); }
static inline void cross3(const double* a, const double* b, double* c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

/* elements.rs:42-181 with the 1-point rules TRIGP1 (xi=eta=1/3, w=1) and
 * QUADGP1 (xi=eta=0, w=4); preprocess.rs:126-153 numbers the points in body
 * element order.  Quad shape derivatives carry 0.25 and detJ another 0.25. */
int64_t oc_collocation(const oc_mesh* m, int64_t body_index, double* cpts) {
    int64_t count = 0;
    for (int64_t e = 0; e < m->nelem; ++e) {
        if (m->body[e] != body_index) continue;
        int t = m->etype[e];
        const int64_t* nd = m->conn + m->conn_off[e];
        int64_t nn = m->conn_off[e + 1] - m->conn_off[e];
        double x[3] = {0, 0, 0}, n[3], area, wt;
        if (t == 5) {
            if (nn < 3) return -1;
            const double third = 1.0 / 3.0;
            double sf[3] = {1.0 - third - third, third, third};
            for (int a = 0; a < 3; ++a) {
                if (nd[a] < 0 || nd[a] >= m->nnodes) return -2;
                const double* X = m->nodes + 3 * nd[a];
                for (int c = 0; c < 3; ++c) x[c] += sf[a] * X[c];
            }
            const double* e0 = m->nodes + 3 * nd[0];
            const double* e1 = m->nodes + 3 * nd[1];
            const double* e2 = m->nodes + 3 * nd[2];
            double a_[3] = {e1[0] - e0[0], e1[1] - e0[1], e1[2] - e0[2]};
            double b_[3] = {e2[0] - e0[0], e2[1] - e0[1], e2[2] - e0[2]};
            cross3(a_, b_, n);
            area = 0.5 * norm3(n);
            wt = 1.0;
        } else if (t == 9) {
            if (nn < 4) return -1;
            static const double dn[4][2] = {{-0.25, -0.25}, {0.25, -0.25}, {0.25, 0.25}, {-0.25, 0.25}};
            double dxi[3] = {0, 0, 0}, deta[3] = {0, 0, 0};
            for (int a = 0; a < 4; ++a) {
                if (nd[a] < 0 || nd[a] >= m->nnodes) return -2;
                const double* X = m->nodes + 3 * nd[a];
                for (int c = 0; c < 3; ++c) {
                    x[c] += 0.25 * X[c];
                    dxi[c] += dn[a][0] * X[c];
                    deta[c] += dn[a][1] * X[c];
                }
            }
            cross3(dxi, deta, n);
            area = 0.25 * norm3(n);
            wt = 4.0;
        } else {
            continue; /* elements.rs:53-56: not numerically integrated, no points */
        }
        if (cpts) {
            double nn_ = norm3(n);
            double* c = cpts + OC_CPT_STRIDE * count;
            c[0] = x[0]; c[1] = x[1]; c[2] = x[2];
            c[3] = n[0] / nn_; c[4] = n[1] / nn_; c[5] = n[2] / nn_;
            c[6] = area; c[7] = wt;
        }
        ++count;
    }
    return count;
}

/* tools.rs:1-10 */
int oc_linspace(double start, double end, int64_t n, double* x) {
    if (n < 1) return 1;
    double dx = (end - start) / (double)(n - 1);
    for (int64_t i = 0; i < n; ++i) x[i] = start;
    for (int64_t i = 1; i < n - 1; ++i) x[i] = start + dx * (double)i;
    x[n - 1] = end;
    return 0;
}

/* tools.rs:12-24 */
int oc_logspace(double start, double end, int64_t n, double* x) {
    if (n < 1) return 1;
    double* xl = (double*)malloc(sizeof(double) * (size_t)n);
    oc_linspace(log10(start), log10(end), n, xl);
    for (int64_t i = 0; i < n; ++i) x[i] = start;
    x[n - 1] = end;
    for (int64_t i = 1; i < n - 1; ++i) x[i] = pow(10.0, xl[i]);
    free(xl);
    return 0;
}

/* ======================================================================= */
/* Problem-level scalars (preprocess.rs:39-74). */
static double omega_of(const oc_problem* p) { return 2.0 * PI * p->frequency; }
static double wavenumber_of(const oc_problem* p) { return omega_of(p) / p->sound_speed; }
static cplx bm_beta(const oc_problem* p) { return I * (1.0 / wavenumber_of(p)); }
static cplx hdiag_of(const oc_problem* p) { return p->problem_type == OC_EXTERIOR ? -0.5 : 0.0; }
static cplx gdiag_of(const oc_problem* p) { return p->method_type == OC_BURTON_MILLER ? 0.5 * bm_beta(p) : 0.0; }

/* influence_matrix.rs:12-37.  x, nx: source (integration) point and normal;
 * y, ny: observation point and normal.  g = e^{ikr}/(4 pi r),
 * h = g (ik - 1/r)(-e_r.n_y); Burton-Miller adds beta*dg, beta*dh. */
static void greens(double k, const double* x, const double* n_x, const double* y,
                   const double* n_y, int bm, cplx beta, cplx* go, cplx* ho) {
    double nnx = norm3(n_x), nny = norm3(n_y);
    double e_nx[3] = {n_x[0] / nnx, n_x[1] / nnx, n_x[2] / nnx};
    double e_ny[3] = {n_y[0] / nny, n_y[1] / nny, n_y[2] / nny};
    double r[3] = {x[0] - y[0], x[1] - y[1], x[2] - y[2]};
    double rdist = norm3(r);
    double e_r[3] = {r[0] / rdist, r[1] / rdist, r[2] / rdist};
    double kr = k * rdist;
    cplx ph = cos(kr) + I * sin(kr);
    double den = 4.0 * PI * rdist;
    cplx g = creal(ph) / den + I * (cimag(ph) / den);
    cplx f1 = -1.0 / rdist + I * k;
    double rdoty = dot3(e_r, e_ny);
    cplx h = (g * f1) * (-rdoty);
    if (bm) {
        double rdotx = dot3(e_r, e_nx);
        cplx gf1 = g * f1;
        cplx dg = gf1 * rdotx;
        cplx t1 = (-f1) * dot3(e_ny, e_nx);
        cplx t2 = ((k * k * rdist + 3.0 * f1) * rdotx) * rdoty;
        cplx dh = ((1.0 / rdist) * g) * (t1 - t2);
        g += beta * dg;
        h += beta * dh;
    }
    *go = g;
    *ho = h;
}

void oc_greens(double k, const double* x, const double* nx, const double* y,
               const double* ny, int bm, double* g, double* h) {
    cplx gg, hh;
    greens(k, x, nx, y, ny, bm, I * (1.0 / k), &gg, &hh);
    g[0] = creal(gg); g[1] = cimag(gg);
    h[0] = creal(hh); h[1] = cimag(hh);
}

/* influence_matrix.rs:39-60: the self term is the static flat disc of equal
 * area (radius b = sqrt(A/pi)); off-diagonal pairs use the collocation normal
 * of row i for h and the source normal of column j for the BM terms. */
static void gh(const oc_problem* p, int64_t i, int64_t j, cplx* go, cplx* ho) {
    int bm = p->method_type == OC_BURTON_MILLER;
    const double* cj = p->cpts + OC_CPT_STRIDE * j;
    if (i == j) {
        double area = cj[6];
        double b = sqrt(area / PI);
        cplx g = 1.0 / (2.0 * PI * b);
        cplx h = 0.0;
        if (bm) h += bm_beta(p) * (-1.0 / (2.0 * PI * (b * b * b)));
        *go = (g * cj[7]) * area;
        *ho = (h * cj[7]) * area;
        return;
    }
    const double* ci = p->cpts + OC_CPT_STRIDE * i;
    cplx g, h;
    greens(wavenumber_of(p), cj, cj + 3, ci, ci + 3, bm, bm_beta(p), &g, &h);
    *go = (g * cj[7]) * cj[6];
    *ho = (h * cj[7]) * cj[6];
}

void oc_gh(const oc_problem* p, int64_t i, int64_t j, double* g, double* h) {
    cplx gg, hh;
    gh(p, i, j, &gg, &hh);
    g[0] = creal(gg); g[1] = cimag(gg);
    h[0] = creal(hh); h[1] = cimag(hh);
}

/* influence_matrix.rs:64-98: H = hdiag I + [h_ij], G = gdiag I + [g_ij].
 * The reference runs one thread-pool task per row (max(nproc/2,2) threads,
 * preprocess.rs:12-17); rows are independent so the result does not depend
 * on the thread count. */
void oc_dense_surface(const oc_problem* p, double* H, double* G, int64_t ld, int nthreads) {
    int64_t n = p->n;
    cplx hd = hdiag_of(p), gd = gdiag_of(p);
#ifdef _OPENMP
    if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#endif
    for (int64_t i = 0; i < n; ++i) {
        for (int64_t j = 0; j < n; ++j) {
            cplx g, h;
            gh(p, i, j, &g, &h);
            cplx h0 = (i == j) ? hd : 0.0, g0 = (i == j) ? gd : 0.0;
            if (H) cput(H, j * ld + i, h0 + h);
            if (G) cput(G, j * ld + i, g0 + g);
        }
    }
    (void)nthreads;
}

/* influence_matrix.rs:101-127: field matrices with the classical kernel, the
 * field point as x and the element as y (source normal n_y). */
void oc_dense_field(const oc_problem* p, double* M, double* L, int64_t ld) {
    double k = wavenumber_of(p);
    double dummy[3] = {0, 0, 0};
    for (int64_t j = 0; j < p->n; ++j) {
        const double* cj = p->cpts + OC_CPT_STRIDE * j;
        for (int64_t i = 0; i < p->nfp; ++i) {
            cplx g, h;
            greens(k, p->field_points + 3 * i, dummy, cj, cj + 3, 0, 0.0, &g, &h);
            cput(M, j * ld + i, (h * cj[7]) * cj[6]);
            cput(L, j * ld + i, (g * cj[7]) * cj[6]);
        }
    }
}

/* influence_matrix.rs:130-146 (system matrix alpha*H + beta*G). */
static void lhs_factors(const oc_problem* p, cplx* a, cplx* b) {
    switch (p->bc_type) {
    case OC_BC_PRESSURE: *a = 0.0; *b = 1.0; break;
    case OC_BC_NORMAL_VELOCITY: *a = 1.0; *b = 0.0; break;
    default: {
        cplx z = p->bc_value[0] + I * p->bc_value[1];
        *a = 1.0;
        *b = (-I * (omega_of(p) * p->mass_density)) / z;
    }
    }
}

/* influence_matrix.rs:149-162 (right-hand side gamma*H + delta*G). */
static void rhs_factors(const oc_problem* p, cplx* a, cplx* b) {
    switch (p->bc_type) {
    case OC_BC_PRESSURE: *a = -1.0; *b = 0.0; break;
    case OC_BC_NORMAL_VELOCITY: *a = 0.0; *b = 1.0; break;
    default: *a = 0.0; *b = 0.0;
    }
}

void oc_lhs_factors(const oc_problem* p, double* alpha, double* beta) {
    cplx a, b;
    lhs_factors(p, &a, &b);
    alpha[0] = creal(a); alpha[1] = cimag(a); beta[0] = creal(b); beta[1] = cimag(b);
}
void oc_rhs_factors(const oc_problem* p, double* gamma, double* delta) {
    cplx a, b;
    rhs_factors(p, &a, &b);
    gamma[0] = creal(a); gamma[1] = cimag(a); delta[0] = creal(b); delta[1] = cimag(b);
}

/* influence_matrix.rs:170-230: one row (ni == 1) or one column (nj == 1) of
 * alpha*H + beta*G including hdiag/gdiag at the first diagonal position. */
int oc_row_or_column(const oc_problem* p, const int64_t* Iv, int64_t ni,
                     const int64_t* Jv, int64_t nj, int side, double* out) {
    if (!((ni == 1) ^ (nj == 1))) return 1;
    cplx al, be;
    if (side) lhs_factors(p, &al, &be); else rhs_factors(p, &al, &be);
    cplx hd = hdiag_of(p), gd = gdiag_of(p);
    int64_t len = (ni == 1) ? nj : ni;
    int diag_done = 0;
    for (int64_t t = 0; t < len; ++t) {
        int64_t i = (ni == 1) ? Iv[0] : Iv[t];
        int64_t j = (ni == 1) ? Jv[t] : Jv[0];
        cplx g, h;
        gh(p, i, j, &g, &h);
        if (i == j && !diag_done) { h += hd; g += gd; diag_done = 1; }
        cput(out, t, be * g + al * h);
    }
    return 0;
}

/* incident_wave.rs:7-63 */
void oc_incident_surface(const oc_problem* p, double* rhs) {
    double k = wavenumber_of(p);
    int bm = p->method_type == OC_BURTON_MILLER;
    cplx beta = bm_beta(p);
    cplx amp = (p->incident_amp[0] + I * p->incident_amp[1]) / (I * (omega_of(p) * p->mass_density));
    double v[3] = {p->incident_vec[0], p->incident_vec[1], p->incident_vec[2]};
    double nv = norm3(v);
    v[0] /= nv; v[1] /= nv; v[2] /= nv; /* spherical origin normalised too (:44) */
    for (int64_t i = 0; i < p->n; ++i) {
        const double* c = p->cpts + OC_CPT_STRIDE * i;
        cplx val;
        if (p->incident_type == OC_PLANE_WAVE) {
            double a = k * dot3(v, c);
            cplx phi = amp * (cos(a) + I * sin(a));
            val = phi;
            if (bm) val += beta * ((phi * (I * k)) * dot3(v, c + 3));
        } else {
            double rv[3] = {c[0] - v[0], c[1] - v[1], c[2] - v[2]};
            double r = norm3(rv);
            double er[3] = {rv[0] / r, rv[1] / r, rv[2] / r};
            cplx ph = amp * (cos(k * r) + I * sin(k * r));
            double den = 4.0 * PI * r;
            cplx phi = creal(ph) / den + I * (cimag(ph) / den);
            val = phi;
            if (bm) val += beta * ((phi * (-1.0 / r + I * k)) * dot3(er, c + 3));
        }
        cput(rhs, i, val);
    }
}

/* incident_wave.rs:66-99 */
void oc_incident_field(const oc_problem* p, double* out) {
    double k = wavenumber_of(p);
    cplx amp = (p->incident_amp[0] + I * p->incident_amp[1]) / (I * (omega_of(p) * p->mass_density));
    double v[3] = {p->incident_vec[0], p->incident_vec[1], p->incident_vec[2]};
    double nv = norm3(v);
    v[0] /= nv; v[1] /= nv; v[2] /= nv;
    for (int64_t i = 0; i < p->nfp; ++i) {
        const double* x = p->field_points + 3 * i;
        cplx val;
        if (p->incident_type == OC_PLANE_WAVE) {
            double a = k * dot3(v, x);
            val = amp * (cos(a) + I * sin(a));
        } else {
            double rv[3] = {x[0] - v[0], x[1] - v[1], x[2] - v[2]};
            double r = norm3(rv);
            cplx ph = amp * (cos(k * r) + I * sin(k * r));
            double den = 4.0 * PI * r;
            val = creal(ph) / den + I * (cimag(ph) / den);
        }
        cput(out, i, val);
    }
}

/* ======================================================================= */
/* Dense complex LU with partial pivoting, nalgebra 0.33.2 `lu()` +
 * `solve_mut` as called by solve.rs:166-171: pivot = first index of maximal
 * |re|+|im| (icamax), unblocked right-looking elimination. */
static double norm1c(cplx z) { return fabs(creal(z)) + fabs(cimag(z)); }

static int lu_factor_inplace(int64_t n, cplx* A, int64_t lda, int64_t* piv) {
    int singular = 0;
    for (int64_t c = 0; c < n; ++c) {
        int64_t pr = c;
        double best = -1.0;
        for (int64_t r = c; r < n; ++r) {
            double v = norm1c(A[c * lda + r]);
            if (v > best) { best = v; pr = r; }
        }
        piv[c] = pr;
        cplx d = A[c * lda + pr];
        if (d == 0.0) { singular = 1; continue; }
        if (pr != c)
            for (int64_t j = 0; j < n; ++j) {
                cplx t = A[j * lda + c];
                A[j * lda + c] = A[j * lda + pr];
                A[j * lda + pr] = t;
            }
        cplx inv = 1.0 / d;
        for (int64_t r = c + 1; r < n; ++r) A[c * lda + r] *= inv;
        for (int64_t j = c + 1; j < n; ++j) {
            cplx a = A[j * lda + c];
            if (a == 0.0) continue;
            cplx* colj = A + j * lda;
            const cplx* colc = A + c * lda;
            for (int64_t r = c + 1; r < n; ++r) colj[r] -= colc[r] * a;
        }
    }
    return singular;
}

static int lu_solve_inplace(int64_t n, const cplx* A, int64_t lda, const int64_t* piv, cplx* b) {
    for (int64_t c = 0; c < n; ++c)
        if (piv[c] != c) { cplx t = b[c]; b[c] = b[piv[c]]; b[piv[c]] = t; }
    for (int64_t c = 0; c < n; ++c) {
        cplx v = b[c];
        for (int64_t r = c + 1; r < n; ++r) b[r] -= A[c * lda + r] * v;
    }
    for (int64_t c = n - 1; c >= 0; --c) {
        cplx d = A[c * lda + c];
        if (d == 0.0) return 1;
        b[c] /= d;
        cplx v = b[c];
        for (int64_t r = 0; r < c; ++r) b[r] -= A[c * lda + r] * v;
    }
    return 0;
}

int oc_lu_solve(int64_t n, const double* A, int64_t lda, double* b) {
    cplx* W = (cplx*)malloc(sizeof(cplx) * (size_t)(n * n > 0 ? n * n : 1));
    int64_t* piv = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    for (int64_t j = 0; j < n; ++j)
        for (int64_t i = 0; i < n; ++i) W[j * n + i] = CPLX(A, j * lda + i);
    int s = lu_factor_inplace(n, W, n, piv);
    int r = lu_solve_inplace(n, W, n, piv, (cplx*)b);
    free(W);
    free(piv);
    return s ? 2 : (r ? 2 : 0);
}

/* ======================================================================= */
/* Restarted GMRES (gmres.rs:35-202) over an abstract operator.  Restart
 * length k = ceil(sqrt(min(max_it, n))), restarts = max_it / k; Arnoldi
 * coefficients use nalgebra dotc(qk1, q_i) = sum conj(qk1) q_i; complex
 * Givens as in LAPACK LAWN 148; stop on the normwise backward error
 * ||r|| / (||A|| ||x|| + ||b||), confirmed with the true residual. */
typedef void (*mv_fn)(void* ctx, const cplx* x, cplx* y); /* y = A x */

static double vnorm(const cplx* v, int64_t n) {
    double s = 0;
    for (int64_t i = 0; i < n; ++i) s += creal(v[i]) * creal(v[i]) + cimag(v[i]) * cimag(v[i]);
    return sqrt(s);
}

static void givens(cplx v1, cplx v2, cplx* cs, cplx* sn) {
    cplx signf = (v1 == 0.0) ? 1.0 : v1 / cabs(v1);
    double n1 = creal(v1) * creal(v1) + cimag(v1) * cimag(v1);
    double n2 = creal(v2) * creal(v2) + cimag(v2) * cimag(v2);
    double r = sqrt(n1 + n2);
    *cs = cabs(v1) / r;
    *sn = signf * conj(v2) / r;
}

static int gmres_generic(int64_t n, mv_fn mv, void* ctx, double anorm, int64_t max_it,
                         double thresh, cplx* x, oc_gmres_report* rep) {
    cplx* b = (cplx*)malloc(sizeof(cplx) * (size_t)n);
    memcpy(b, x, sizeof(cplx) * (size_t)n);
    for (int64_t i = 0; i < n; ++i) x[i] = 0.0;
    if (max_it <= 0) max_it = 1000;
    if (max_it > n) max_it = n;
    if (thresh <= 0.0) thresh = 1e-5;
    int64_t m = (int64_t)ceil(sqrt((double)max_it));
    int64_t restarts = max_it / m;
    cplx* r = (cplx*)malloc(sizeof(cplx) * (size_t)n);
    cplx* ax = (cplx*)malloc(sizeof(cplx) * (size_t)n);
    cplx* Q = (cplx*)malloc(sizeof(cplx) * (size_t)(n * (m + 1)));
    cplx* Hm = (cplx*)malloc(sizeof(cplx) * (size_t)((m + 1) * m));
    cplx* hk1 = (cplx*)malloc(sizeof(cplx) * (size_t)(m + 1));
    cplx* beta = (cplx*)malloc(sizeof(cplx) * (size_t)(m + 1));
    cplx* cs = (cplx*)malloc(sizeof(cplx) * (size_t)m);
    cplx* sn = (cplx*)malloc(sizeof(cplx) * (size_t)m);
    cplx* hk = (cplx*)malloc(sizeof(cplx) * (size_t)(m * m));
    cplx* y = (cplx*)malloc(sizeof(cplx) * (size_t)m);
    int64_t* piv = (int64_t*)malloc(sizeof(int64_t) * (size_t)m);
    int64_t num_mv = 0;
    int flag = 0;
    double error = 0;
    double bnorm = vnorm(b, n);
    int64_t rs;
    for (rs = 0; rs < restarts; ++rs) {
        flag = 0;
        mv(ctx, x, ax); ++num_mv;
        for (int64_t i = 0; i < n; ++i) r[i] = b[i] - ax[i];
        double rn = vnorm(r, n);
        error = rn / (anorm * vnorm(x, n) + bnorm);
        for (int64_t i = 0; i < m; ++i) { cs[i] = 0; sn[i] = 0; }
        memset(Q, 0, sizeof(cplx) * (size_t)(n * (m + 1)));
        memset(Hm, 0, sizeof(cplx) * (size_t)((m + 1) * m));
        for (int64_t i = 0; i < n; ++i) Q[i] = creal(r[i]) / rn + I * (cimag(r[i]) / rn);
        for (int64_t i = 0; i <= m; ++i) beta[i] = 0;
        beta[0] = rn;
        for (int64_t k = 0; k < m; ++k) {
            /* arnoldi (gmres.rs:158-176) */
            cplx* qk1 = Q + (k + 1) * n;
            mv(ctx, Q + k * n, qk1); ++num_mv;
            for (int64_t i = 0; i <= m; ++i) hk1[i] = 0;
            for (int64_t i = 0; i <= k; ++i) {
                const cplx* qi = Q + i * n;
                cplx s = 0;
                for (int64_t l = 0; l < n; ++l) s += conj(qk1[l]) * qi[l];
                hk1[i] = s;
                for (int64_t l = 0; l < n; ++l) qk1[l] += (-s) * qi[l];
            }
            hk1[k + 1] = vnorm(qk1, n);
            cplx scale = 1.0 / hk1[k + 1];
            for (int64_t l = 0; l < n; ++l) qk1[l] *= scale;
            /* apply_givens_rotation (gmres.rs:178-190) */
            for (int64_t i = 0; i < k; ++i) {
                cplx t = cs[i] * hk1[i] + sn[i] * hk1[i + 1];
                hk1[i + 1] = -conj(sn[i]) * hk1[i] + cs[i] * hk1[i + 1];
                hk1[i] = t;
            }
            givens(hk1[k], hk1[k + 1], &cs[k], &sn[k]);
            hk1[k] = cs[k] * hk1[k] + sn[k] * hk1[k + 1];
            hk1[k + 1] = 0;
            for (int64_t i = 0; i < k + 2; ++i) Hm[k * (m + 1) + i] = hk1[i];
            beta[k + 1] = -conj(sn[k]) * beta[k];
            beta[k] *= cs[k];
            error = cabs(beta[k + 1]) / (anorm * vnorm(x, n) + bnorm);
            if (error < thresh || k == m - 1) {
                /* get_x (gmres.rs:146-157): y = H_k^-1 beta_k, x += Q_k y */
                int64_t kk = k + 1;
                for (int64_t j = 0; j < kk; ++j)
                    for (int64_t i = 0; i < kk; ++i) hk[j * kk + i] = Hm[j * (m + 1) + i];
                for (int64_t i = 0; i < kk; ++i) y[i] = beta[i];
                lu_factor_inplace(kk, hk, kk, piv);
                lu_solve_inplace(kk, hk, kk, piv, y);
                for (int64_t j = 0; j < kk; ++j) {
                    cplx yj = y[j];
                    const cplx* qj = Q + j * n;
                    for (int64_t l = 0; l < n; ++l) x[l] += qj[l] * yj;
                }
                mv(ctx, x, ax); ++num_mv;
                for (int64_t i = 0; i < n; ++i) r[i] = b[i] - ax[i];
                error = vnorm(r, n) / (anorm * vnorm(x, n) + bnorm);
                if (error < thresh) { flag = 1; break; }
            }
            if (k == m - 1) flag = 2;
        }
        if (flag == 1) break;
    }
    if (rep) {
        rep->num_mv = num_mv;
        rep->restarts = rs < restarts ? rs + 1 : restarts;
        rep->error = error;
        rep->flag = flag;
    }
    free(b); free(r); free(ax); free(Q); free(Hm); free(hk1); free(beta);
    free(cs); free(sn); free(hk); free(y); free(piv);
    return flag == 1 ? 0 : 3;
}

typedef struct { int64_t n; const cplx* A; int64_t lda; } dense_ctx;
static void dense_mv(void* c, const cplx* x, cplx* y) {
    const dense_ctx* d = (const dense_ctx*)c;
    for (int64_t i = 0; i < d->n; ++i) y[i] = 0;
    for (int64_t j = 0; j < d->n; ++j) {
        cplx xj = x[j];
        const cplx* col = d->A + j * d->lda;
        for (int64_t i = 0; i < d->n; ++i) y[i] += col[i] * xj;
    }
}

static double frob(int64_t m, int64_t n, const cplx* A, int64_t lda) {
    double s = 0;
    for (int64_t j = 0; j < n; ++j)
        for (int64_t i = 0; i < m; ++i) {
            cplx v = A[j * lda + i];
            s += creal(v) * creal(v) + cimag(v) * cimag(v);
        }
    return sqrt(s);
}

int oc_gmres_dense(int64_t n, const double* A, int64_t lda, int64_t max_it, double tol,
                   double* x, oc_gmres_report* rep) {
    dense_ctx d = {n, (const cplx*)A, lda};
    return gmres_generic(n, dense_mv, &d, frob(n, n, (const cplx*)A, lda), max_it, tol, (cplx*)x, rep);
}

/* ======================================================================= */
/* Cluster tree (cluster.rs:35-105): bisect the bounding box at the midpoint
 * of its longest axis (<= goes to the first son) until a cluster holds at
 * most leaf points; diameter = box diagonal, distance = box gap. */
typedef struct cl_node {
    double lo[3], hi[3], diam;
    int64_t* idx;
    int64_t cnt;
    struct cl_node* son[2];
} cl_node;

static cl_node* cluster_build(const double* pts, int64_t stride, int64_t* idx, int64_t cnt,
                              int64_t leaf, int depth, int* err) {
    cl_node* c = (cl_node*)calloc(1, sizeof(cl_node));
    c->idx = idx;
    c->cnt = cnt;
    for (int d = 0; d < 3; ++d) { c->lo[d] = INFINITY; c->hi[d] = -INFINITY; }
    for (int64_t t = 0; t < cnt; ++t)
        for (int d = 0; d < 3; ++d) {
            double v = pts[stride * idx[t] + d];
            c->lo[d] = fmin(v, c->lo[d]);
            c->hi[d] = fmax(v, c->hi[d]);
        }
    double s = 0;
    for (int d = 0; d < 3; ++d) s += (c->hi[d] - c->lo[d]) * (c->hi[d] - c->lo[d]);
    c->diam = sqrt(s);
    if (cnt <= leaf) return c;
    if (depth > 200) { *err = 1; return c; }
    int jmax = 0;
    double diff = 0;
    for (int d = 0; d < 3; ++d) {
        double e = c->hi[d] - c->lo[d];
        if (e > diff) { jmax = d; diff = e; }
    }
    double gamma = 0.5 * (c->lo[jmax] + c->hi[jmax]);
    /* stable partition into a fresh buffer keeps each son's original order */
    int64_t* tmp = (int64_t*)malloc(sizeof(int64_t) * (size_t)cnt);
    int64_t n1 = 0, n2 = 0;
    for (int64_t t = 0; t < cnt; ++t)
        if (pts[stride * idx[t] + jmax] <= gamma) tmp[n1++] = idx[t];
    for (int64_t t = 0; t < cnt; ++t)
        if (!(pts[stride * idx[t] + jmax] <= gamma)) tmp[n1 + n2++] = idx[t];
    memcpy(idx, tmp, sizeof(int64_t) * (size_t)cnt);
    free(tmp);
    if (n1 == 0 || n2 == 0) { *err = 1; return c; }
    c->son[0] = cluster_build(pts, stride, idx, n1, leaf, depth + 1, err);
    c->son[1] = cluster_build(pts, stride, idx + n1, n2, leaf, depth + 1, err);
    return c;
}

static void cluster_free(cl_node* c) {
    if (!c) return;
    cluster_free(c->son[0]);
    cluster_free(c->son[1]);
    free(c);
}

static double cluster_dist(const cl_node* a, const cl_node* b) {
    double s = 0;
    for (int d = 0; d < 3; ++d) {
        double t1 = fmax(0.0, a->lo[d] - b->hi[d]);
        double t2 = fmax(0.0, b->lo[d] - a->hi[d]);
        s += t1 * t1;
        s += t2 * t2;
    }
    return sqrt(s);
}

/* Block tree (block.rs:38-55) flattened depth-first (block.rs:76-93). */
typedef struct {
    int64_t n, cap;
    const cl_node** r;
    const cl_node** c;
    int32_t* adm;
} blk_vec;

static void blk_push(blk_vec* v, const cl_node* r, const cl_node* c, int adm) {
    if (v->n == v->cap) {
        v->cap = v->cap ? 2 * v->cap : 64;
        v->r = (const cl_node**)realloc(v->r, sizeof(void*) * (size_t)v->cap);
        v->c = (const cl_node**)realloc(v->c, sizeof(void*) * (size_t)v->cap);
        v->adm = (int32_t*)realloc(v->adm, sizeof(int32_t) * (size_t)v->cap);
    }
    v->r[v->n] = r; v->c[v->n] = c; v->adm[v->n] = adm; v->n++;
}

static void block_recurse(const cl_node* r, const cl_node* c, double eta, blk_vec* out) {
    int adm = fmin(r->diam, c->diam) <= eta * cluster_dist(r, c);
    int rleaf = r->son[0] == NULL, cleaf = c->son[0] == NULL;
    if (adm || rleaf || cleaf) { blk_push(out, r, c, adm); return; }
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b) block_recurse(r->son[a], c->son[b], eta, out);
}

int oc_block_list(int64_t n, const double* pts, int64_t stride, int64_t leaf, double eta,
                  oc_blocklist* out) {
    memset(out, 0, sizeof *out);
    int64_t* idx = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    for (int64_t i = 0; i < n; ++i) idx[i] = i;
    int err = 0;
    cl_node* root = cluster_build(pts, stride, idx, n, leaf, 0, &err);
    if (err) { cluster_free(root); free(idx); return 1; }
    blk_vec v = {0};
    block_recurse(root, root, eta, &v);
    out->nblocks = v.n;
    out->root_diameter = root->diam;
    out->row_off = (int64_t*)malloc(sizeof(int64_t) * (size_t)(v.n + 1));
    out->col_off = (int64_t*)malloc(sizeof(int64_t) * (size_t)(v.n + 1));
    out->admissible = (int32_t*)malloc(sizeof(int32_t) * (size_t)(v.n ? v.n : 1));
    int64_t tr = 0, tc = 0;
    out->row_off[0] = out->col_off[0] = 0;
    for (int64_t b = 0; b < v.n; ++b) {
        tr += v.r[b]->cnt; tc += v.c[b]->cnt;
        out->row_off[b + 1] = tr; out->col_off[b + 1] = tc;
        out->admissible[b] = v.adm[b];
    }
    out->rows = (int64_t*)malloc(sizeof(int64_t) * (size_t)(tr ? tr : 1));
    out->cols = (int64_t*)malloc(sizeof(int64_t) * (size_t)(tc ? tc : 1));
    for (int64_t b = 0; b < v.n; ++b) {
        memcpy(out->rows + out->row_off[b], v.r[b]->idx, sizeof(int64_t) * (size_t)v.r[b]->cnt);
        memcpy(out->cols + out->col_off[b], v.c[b]->idx, sizeof(int64_t) * (size_t)v.c[b]->cnt);
    }
    free(v.r); free(v.c); free(v.adm);
    cluster_free(root);
    free(idx);
    return 0;
}

void oc_blocklist_free(oc_blocklist* b) {
    free(b->row_off); free(b->rows); free(b->col_off); free(b->cols); free(b->admissible);
    memset(b, 0, sizeof *b);
}

/* block.rs:104-115 inspects block_tree.children[1].children[1].children[1]. */
typedef struct bt_node { int adm; int nch; struct bt_node* ch[4]; } bt_node;
static bt_node* bt_build(const cl_node* r, const cl_node* c, double eta) {
    bt_node* t = (bt_node*)calloc(1, sizeof(bt_node));
    t->adm = fmin(r->diam, c->diam) <= eta * cluster_dist(r, c);
    if (!(t->adm || r->son[0] == NULL || c->son[0] == NULL)) {
        for (int a = 0; a < 2; ++a)
            for (int b = 0; b < 2; ++b) t->ch[t->nch++] = bt_build(r->son[a], c->son[b], eta);
    }
    return t;
}
static void bt_free(bt_node* t) {
    if (!t) return;
    for (int i = 0; i < t->nch; ++i) bt_free(t->ch[i]);
    free(t);
}

int oc_block_tree_path_admissible(int64_t n, const double* pts, int64_t stride, int64_t leaf,
                                  double eta, const int32_t* path, int depth) {
    int64_t* idx = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    for (int64_t i = 0; i < n; ++i) idx[i] = i;
    int err = 0;
    cl_node* root = cluster_build(pts, stride, idx, n, leaf, 0, &err);
    bt_node* t = bt_build(root, root, eta);
    bt_node* cur = t;
    int res = -1;
    for (int d = 0; d < depth && cur; ++d) cur = (path[d] < cur->nch) ? cur->ch[path[d]] : NULL;
    if (cur) res = cur->adm;
    bt_free(t);
    cluster_free(root);
    free(idx);
    return res;
}

/* ======================================================================= */
/* Complex Householder QR (m x r, m >= r) returning thin Q (m x r) and R (r x r),
 * and a one-sided Jacobi SVD; together they restate the nalgebra QR/SVD used
 * by aca.rs:137-179.  Any backward-stable QR/SVD yields the same truncated
 * U V^T, which is what the reference's results depend on. */
static void house_qr(int64_t m, int64_t r, const cplx* A, cplx* Q, cplx* R) {
    cplx* W = (cplx*)malloc(sizeof(cplx) * (size_t)(m * r));
    memcpy(W, A, sizeof(cplx) * (size_t)(m * r));
    cplx* V = (cplx*)calloc((size_t)(m * r), sizeof(cplx));
    cplx* tau = (cplx*)calloc((size_t)r, sizeof(cplx));
    for (int64_t k = 0; k < r; ++k) {
        double s = 0;
        for (int64_t i = k; i < m; ++i) s += creal(W[k * m + i]) * creal(W[k * m + i]) + cimag(W[k * m + i]) * cimag(W[k * m + i]);
        double nx = sqrt(s);
        cplx x0 = W[k * m + k];
        cplx ph = (cabs(x0) == 0) ? 1.0 : x0 / cabs(x0);
        cplx alpha = -ph * nx;
        cplx* v = V + k * m;
        for (int64_t i = k; i < m; ++i) v[i] = W[k * m + i];
        v[k] -= alpha;
        double vn = 0;
        for (int64_t i = k; i < m; ++i) vn += creal(v[i]) * creal(v[i]) + cimag(v[i]) * cimag(v[i]);
        if (vn == 0) { tau[k] = 0; continue; }
        tau[k] = 2.0 / vn;
        for (int64_t j = k; j < r; ++j) {
            cplx d = 0;
            for (int64_t i = k; i < m; ++i) d += conj(v[i]) * W[j * m + i];
            d *= tau[k];
            for (int64_t i = k; i < m; ++i) W[j * m + i] -= v[i] * d;
        }
    }
    for (int64_t j = 0; j < r; ++j)
        for (int64_t i = 0; i < r; ++i) R[j * r + i] = (i <= j) ? W[j * m + i] : 0.0;
    /* Q = H_0 H_1 ... H_{r-1} applied to the first r columns of I */
    for (int64_t j = 0; j < r; ++j)
        for (int64_t i = 0; i < m; ++i) Q[j * m + i] = (i == j) ? 1.0 : 0.0;
    for (int64_t k = r - 1; k >= 0; --k) {
        if (tau[k] == 0.0) continue;
        const cplx* v = V + k * m;
        for (int64_t j = 0; j < r; ++j) {
            cplx d = 0;
            for (int64_t i = k; i < m; ++i) d += conj(v[i]) * Q[j * m + i];
            d *= tau[k];
            for (int64_t i = k; i < m; ++i) Q[j * m + i] -= v[i] * d;
        }
    }
    free(W); free(V); free(tau);
}

/* One-sided Jacobi SVD of a square r x r complex matrix: A = W S Vh with
 * singular values sorted descending. */
static void jacobi_svd(int64_t r, const cplx* A, cplx* W, double* S, cplx* Vh) {
    cplx* U = (cplx*)malloc(sizeof(cplx) * (size_t)(r * r));
    cplx* V = (cplx*)malloc(sizeof(cplx) * (size_t)(r * r));
    memcpy(U, A, sizeof(cplx) * (size_t)(r * r));
    for (int64_t j = 0; j < r; ++j)
        for (int64_t i = 0; i < r; ++i) V[j * r + i] = (i == j) ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 60; ++sweep) {
        double off = 0;
        for (int64_t p = 0; p < r; ++p)
            for (int64_t q = p + 1; q < r; ++q) {
                double a = 0, b = 0;
                cplx c = 0;
                for (int64_t i = 0; i < r; ++i) {
                    a += creal(U[p * r + i]) * creal(U[p * r + i]) + cimag(U[p * r + i]) * cimag(U[p * r + i]);
                    b += creal(U[q * r + i]) * creal(U[q * r + i]) + cimag(U[q * r + i]) * cimag(U[q * r + i]);
                    c += conj(U[p * r + i]) * U[q * r + i];
                }
                double ac = cabs(c);
                if (ac == 0 || ac <= 1e-15 * sqrt(a * b)) continue;
                off = fmax(off, ac / sqrt(a * b));
                double zeta = (b - a) / (2.0 * ac);
                double t = (zeta >= 0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
                double cs = 1.0 / sqrt(1.0 + t * t), sn = cs * t;
                cplx e = c / ac; /* phase */
                for (int64_t i = 0; i < r; ++i) {
                    cplx up = U[p * r + i], uq = U[q * r + i];
                    U[p * r + i] = cs * up - sn * conj(e) * uq;
                    U[q * r + i] = sn * e * up + cs * uq;
                    cplx vp = V[p * r + i], vq = V[q * r + i];
                    V[p * r + i] = cs * vp - sn * conj(e) * vq;
                    V[q * r + i] = sn * e * vp + cs * vq;
                }
            }
        if (off < 1e-15) break;
    }
    /* singular values = column norms; sort descending */
    int64_t* ord = (int64_t*)malloc(sizeof(int64_t) * (size_t)r);
    double* sv = (double*)malloc(sizeof(double) * (size_t)r);
    for (int64_t j = 0; j < r; ++j) { sv[j] = vnorm(U + j * r, r); ord[j] = j; }
    for (int64_t a = 0; a < r; ++a)
        for (int64_t b2 = a + 1; b2 < r; ++b2)
            if (sv[ord[b2]] > sv[ord[a]]) { int64_t t = ord[a]; ord[a] = ord[b2]; ord[b2] = t; }
    for (int64_t jj = 0; jj < r; ++jj) {
        int64_t j = ord[jj];
        S[jj] = sv[j];
        for (int64_t i = 0; i < r; ++i) {
            W[jj * r + i] = sv[j] > 0 ? U[j * r + i] / sv[j] : (i == jj ? 1.0 : 0.0);
            Vh[i * r + jj] = conj(V[j * r + i]); /* row jj of Vh = V[:,j]^H */
        }
    }
    free(U); free(V); free(ord); free(sv);
}

/* ACA with partial pivoting (aca.rs:57-136) followed by QR+SVD recompression
 * (aca.rs:137-179) and the ab-initio norm estimate (aca.rs:212-222). */
typedef struct {
    int64_t m, n, rank, cap;
    cplx* U; /* m x cap */
    cplx* V; /* n x cap */
    double norm;
} aca_t;

typedef struct {
    oc_rowcol_fn gen;
    void* ctx;
    const int64_t* rows;
    const int64_t* cols;
    int64_t m, n;
    int64_t* scratch;
} aca_src;

static void aca_row(const aca_src* s, int64_t i, cplx* out) {
    int64_t gi = s->rows ? s->rows[i] : i;
    if (s->cols) s->gen(s->ctx, &gi, 1, s->cols, s->n, (double*)out);
    else {
        for (int64_t j = 0; j < s->n; ++j) s->scratch[j] = j;
        s->gen(s->ctx, &gi, 1, s->scratch, s->n, (double*)out);
    }
}
static void aca_col(const aca_src* s, int64_t j, cplx* out) {
    int64_t gj = s->cols ? s->cols[j] : j;
    if (s->rows) s->gen(s->ctx, s->rows, s->m, &gj, 1, (double*)out);
    else {
        for (int64_t i = 0; i < s->m; ++i) s->scratch[i] = i;
        s->gen(s->ctx, s->scratch, s->m, &gj, 1, (double*)out);
    }
}

static void aca_res_row(const aca_t* a, const aca_src* s, int64_t i, cplx* r) {
    aca_row(s, i, r);
    for (int64_t k = 0; k < a->rank; ++k) {
        cplx f = -a->U[k * a->m + i];
        const cplx* v = a->V + k * a->n;
        for (int64_t j = 0; j < a->n; ++j) r[j] += v[j] * f;
    }
}
static void aca_res_col(const aca_t* a, const aca_src* s, int64_t j, cplx* r) {
    aca_col(s, j, r);
    for (int64_t k = 0; k < a->rank; ++k) {
        cplx f = -a->V[k * a->n + j];
        const cplx* u = a->U + k * a->m;
        for (int64_t i = 0; i < a->m; ++i) r[i] += u[i] * f;
    }
}

static int64_t idx_max_excl(const cplx* v, int64_t len, const char* excl) {
    int64_t index = len;
    double best = -1.0;
    for (int64_t i = 0; i < len; ++i) {
        if (excl[i]) continue;
        double a = cabs(v[i]);
        if (best < a) { index = i; best = a; }
    }
    return index;
}

static cplx dotu(const cplx* a, const cplx* b, int64_t n) {
    cplx s = 0;
    for (int64_t i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}
static double nsq(const cplx* a, int64_t n) {
    double s = 0;
    for (int64_t i = 0; i < n; ++i) s += creal(a[i]) * creal(a[i]) + cimag(a[i]) * cimag(a[i]);
    return s;
}

static void random_index_exclude(int64_t* i, int64_t n, const char* excl, oc_stdrng* rng) {
    if (excl[*i]) {
        *i = (int64_t)oc_uniform_usize_incl(rng, 0, (uint64_t)(n - 1));
        for (int64_t t = 0; t < n - 1; ++t) {
            *i = (*i + 1) % n;
            if (!excl[*i]) break;
        }
    }
}

static void aca_decompose(aca_t* a, const aca_src* s, double tol) {
    int64_t m = a->m, n = a->n;
    int64_t nr = m < n ? m : n;
    a->cap = nr;
    a->U = (cplx*)calloc((size_t)(m * nr), sizeof(cplx));
    a->V = (cplx*)calloc((size_t)(n * nr), sizeof(cplx));
    a->rank = 0;
    oc_stdrng rng;
    oc_stdrng_seed(&rng, 10);
    int64_t iref = (int64_t)oc_uniform_usize_incl(&rng, 0, (uint64_t)(nr - 1));
    int64_t jref = (int64_t)oc_uniform_usize_incl(&rng, 0, (uint64_t)(nr - 1));
    char* iex = (char*)calloc((size_t)m + 1, 1);
    char* jex = (char*)calloc((size_t)n + 1, 1);
    cplx* riref = (cplx*)malloc(sizeof(cplx) * (size_t)n);
    cplx* rjref = (cplx*)malloc(sizeof(cplx) * (size_t)m);
    cplx* ristar = (cplx*)malloc(sizeof(cplx) * (size_t)n);
    cplx* rjstar = (cplx*)malloc(sizeof(cplx) * (size_t)m);
    aca_res_row(a, s, iref, riref);
    aca_res_col(a, s, jref, rjref);
    double total = 0;
    for (int64_t k = 0; k < nr; ++k) {
        int64_t jstar = idx_max_excl(riref, n, jex);
        double jval = cabs(riref[jstar]);
        int64_t istar = idx_max_excl(rjref, m, iex);
        double ival = cabs(rjref[istar]);
        if (ival > jval) {
            aca_res_row(a, s, istar, ristar);
            jstar = idx_max_excl(ristar, n, jex);
            aca_res_col(a, s, jstar, rjstar);
        } else {
            aca_res_col(a, s, jstar, rjstar);
            istar = idx_max_excl(rjstar, m, iex);
            aca_res_row(a, s, istar, ristar);
        }
        iex[istar] = 1;
        jex[jstar] = 1;
        cplx f = 1.0 / ristar[jstar];
        for (int64_t j = 0; j < n; ++j) ristar[j] *= f;
        memcpy(a->U + k * m, rjstar, sizeof(cplx) * (size_t)m);
        memcpy(a->V + k * n, ristar, sizeof(cplx) * (size_t)n);
        a->rank = k + 1;
        /* update_norm_estimate (aca.rs:224-241) */
        const cplx* u = a->U + k * m;
        const cplx* v = a->V + k * n;
        double nk = nsq(u, m) * nsq(v, n);
        total += nk;
        for (int64_t t = 0; t < k; ++t)
            total += 2.0 * cabs(dotu(a->U + t * m, u, m)) * cabs(dotu(a->V + t * n, v, n));
        double step = sqrt(nk) / sqrt(total);
        if (step < tol / 50.0) break;
        if (iref == istar) {
            random_index_exclude(&iref, nr, iex, &rng);
            aca_res_row(a, s, iref, riref);
        } else {
            cplx g = -u[iref];
            for (int64_t j = 0; j < n; ++j) riref[j] += v[j] * g;
        }
        if (jref == jstar) {
            random_index_exclude(&jref, nr, jex, &rng);
            aca_res_col(a, s, jref, rjref);
        } else {
            cplx g = -v[jref];
            for (int64_t i = 0; i < m; ++i) rjref[i] += u[i] * g;
        }
    }
    a->norm = sqrt(total);
    free(iex); free(jex); free(riref); free(rjref); free(ristar); free(rjstar);

    /* svd_recompression (aca.rs:137-179) */
    int64_t r = a->rank;
    cplx* Qu = (cplx*)malloc(sizeof(cplx) * (size_t)(m * r));
    cplx* Ru = (cplx*)malloc(sizeof(cplx) * (size_t)(r * r));
    cplx* Qv = (cplx*)malloc(sizeof(cplx) * (size_t)(n * r));
    cplx* Rv = (cplx*)malloc(sizeof(cplx) * (size_t)(r * r));
    house_qr(m, r, a->U, Qu, Ru);
    house_qr(n, r, a->V, Qv, Rv);
    cplx* RR = (cplx*)calloc((size_t)(r * r), sizeof(cplx));
    for (int64_t j = 0; j < r; ++j)
        for (int64_t l = 0; l < r; ++l) {
            cplx rv = Rv[l * r + j]; /* (R_v^T)[l][j] = R_v[j][l] */
            for (int64_t i = 0; i < r; ++i) RR[j * r + i] += Ru[l * r + i] * rv;
        }
    cplx* W = (cplx*)malloc(sizeof(cplx) * (size_t)(r * r));
    cplx* Vh = (cplx*)malloc(sizeof(cplx) * (size_t)(r * r));
    double* S = (double*)malloc(sizeof(double) * (size_t)r);
    jacobi_svd(r, RR, W, S, Vh);
    int64_t index = 0;
    double sum = 0;
    for (int64_t t = 0; t < r; ++t) {
        sum += S[t];
        if (S[t] < tol * sum) break;
        index++;
    }
    index = index + 1 < r ? index + 1 : r;
    if (index < 1) index = 1;
    for (int64_t t = 0; t < index; ++t) {
        cplx* u = a->U + t * m;
        cplx* v = a->V + t * n;
        for (int64_t i = 0; i < m; ++i) {
            cplx acc = 0;
            for (int64_t l = 0; l < r; ++l) acc += Qu[l * m + i] * W[t * r + l];
            u[i] = S[t] * acc;
        }
        for (int64_t i = 0; i < n; ++i) {
            cplx acc = 0;
            for (int64_t l = 0; l < r; ++l) acc += Qv[l * n + i] * Vh[l * r + t]; /* z = Vh^T */
            v[i] = acc;
        }
    }
    a->rank = index;
    free(Qu); free(Ru); free(Qv); free(Rv); free(RR); free(W); free(Vh); free(S);
    /* calculate_norm_estimate (aca.rs:212-222) */
    double tot = 0;
    for (int64_t i = 0; i < a->rank; ++i) {
        const cplx* ui = a->U + i * m;
        const cplx* vi = a->V + i * n;
        tot += nsq(ui, m) * nsq(vi, n);
        for (int64_t j = 0; j < i; ++j)
            tot += 2.0 * cabs(dotu(ui, a->U + j * m, m)) * cabs(dotu(vi, a->V + j * n, n));
    }
    a->norm = sqrt(tot);
}

int64_t oc_aca(int64_t m, int64_t n, double tol, oc_rowcol_fn gen, void* ctx,
               double* U, double* V, double* norm_est) {
    aca_src s = {gen, ctx, NULL, NULL, m, n, NULL};
    s.scratch = (int64_t*)malloc(sizeof(int64_t) * (size_t)(m > n ? m : n));
    aca_t a = {m, n, 0, 0, NULL, NULL, 0};
    aca_decompose(&a, &s, tol);
    if (U) memcpy(U, a.U, sizeof(cplx) * (size_t)(m * a.rank));
    if (V) memcpy(V, a.V, sizeof(cplx) * (size_t)(n * a.rank));
    if (norm_est) *norm_est = a.norm;
    int64_t r = a.rank;
    free(a.U); free(a.V); free(s.scratch);
    return r;
}

/* ======================================================================= */
/* H-matrix (h_matrix.rs:110-247): leaves of the flattened block tree are
 * either ACA low-rank (admissible) or dense (inadmissible).  gemv scales b
 * by beta, then gathers x, multiplies and scatter-adds alpha*(block x). */
struct oc_hmatrix {
    int64_t n;
    double norm;
    oc_blocklist bl;
    aca_t* lr;     /* per block, valid for admissible */
    cplx** dense;  /* per block, valid for inadmissible (m x n col-major) */
};

oc_hmatrix* oc_hmatrix_build(int64_t n, const double* pts, int64_t stride, int64_t leaf,
                             double eta, double tol, oc_rowcol_fn gen, void* ctx) {
    oc_hmatrix* h = (oc_hmatrix*)calloc(1, sizeof(oc_hmatrix));
    h->n = n;
    if (oc_block_list(n, pts, stride, leaf, eta, &h->bl)) { free(h); return NULL; }
    int64_t nb = h->bl.nblocks;
    h->lr = (aca_t*)calloc((size_t)nb, sizeof(aca_t));
    h->dense = (cplx**)calloc((size_t)nb, sizeof(cplx*));
    int64_t maxd = 1;
    for (int64_t b = 0; b < nb; ++b) {
        int64_t m = h->bl.row_off[b + 1] - h->bl.row_off[b];
        int64_t c = h->bl.col_off[b + 1] - h->bl.col_off[b];
        if (m > maxd) maxd = m;
        if (c > maxd) maxd = c;
    }
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (int64_t b = 0; b < nb; ++b) {
        const int64_t* rows = h->bl.rows + h->bl.row_off[b];
        const int64_t* cols = h->bl.cols + h->bl.col_off[b];
        int64_t m = h->bl.row_off[b + 1] - h->bl.row_off[b];
        int64_t c = h->bl.col_off[b + 1] - h->bl.col_off[b];
        if (h->bl.admissible[b]) {
            aca_src s = {gen, ctx, rows, cols, m, c, NULL};
            h->lr[b].m = m;
            h->lr[b].n = c;
            aca_decompose(&h->lr[b], &s, tol);
        } else {
            cplx* D = (cplx*)malloc(sizeof(cplx) * (size_t)(m * c));
            cplx* rowbuf = (cplx*)malloc(sizeof(cplx) * (size_t)c);
            for (int64_t i = 0; i < m; ++i) {
                gen(ctx, rows + i, 1, cols, c, (double*)rowbuf);
                for (int64_t j = 0; j < c; ++j) D[j * m + i] = rowbuf[j];
            }
            free(rowbuf);
            h->dense[b] = D;
        }
    }
    /* update_norm (h_matrix.rs:189-196): sum of block norms */
    double s = 0;
    for (int64_t b = 0; b < nb; ++b) {
        int64_t m = h->bl.row_off[b + 1] - h->bl.row_off[b];
        int64_t c = h->bl.col_off[b + 1] - h->bl.col_off[b];
        if (!h->bl.admissible[b]) s += frob(m, c, h->dense[b], m);
    }
    for (int64_t b = 0; b < nb; ++b)
        if (h->bl.admissible[b]) s += h->lr[b].norm;
    h->norm = s;
    return h;
}

void oc_hmatrix_free(oc_hmatrix* h) {
    if (!h) return;
    for (int64_t b = 0; b < h->bl.nblocks; ++b) {
        free(h->lr[b].U); free(h->lr[b].V); free(h->dense[b]);
    }
    free(h->lr); free(h->dense);
    oc_blocklist_free(&h->bl);
    free(h);
}

double oc_hmatrix_norm(const oc_hmatrix* h) { return h->norm; }
int64_t oc_hmatrix_num_blocks(const oc_hmatrix* h) { return h->bl.nblocks; }

static void hm_gemv(const oc_hmatrix* h, cplx alpha, const cplx* x, cplx beta, cplx* b) {
    if (beta != 1.0) for (int64_t i = 0; i < h->n; ++i) b[i] *= beta;
    int64_t nb = h->bl.nblocks;
    cplx* x1 = (cplx*)malloc(sizeof(cplx) * (size_t)(h->n + 1));
    cplx* b1 = (cplx*)malloc(sizeof(cplx) * (size_t)(h->n + 1));
    for (int pass = 0; pass < 2; ++pass)
        for (int64_t blk = 0; blk < nb; ++blk) {
            int adm = h->bl.admissible[blk];
            if (adm != pass) continue; /* inadmissible blocks first (h_matrix.rs:228-233) */
            const int64_t* rows = h->bl.rows + h->bl.row_off[blk];
            const int64_t* cols = h->bl.cols + h->bl.col_off[blk];
            int64_t m = h->bl.row_off[blk + 1] - h->bl.row_off[blk];
            int64_t c = h->bl.col_off[blk + 1] - h->bl.col_off[blk];
            for (int64_t j = 0; j < c; ++j) x1[j] = x[cols[j]];
            for (int64_t i = 0; i < m; ++i) b1[i] = 0;
            if (!adm) {
                const cplx* D = h->dense[blk];
                for (int64_t j = 0; j < c; ++j) {
                    cplx f = alpha * x1[j];
                    for (int64_t i = 0; i < m; ++i) b1[i] += D[j * m + i] * f;
                }
            } else {
                const aca_t* a = &h->lr[blk];
                for (int64_t k = 0; k < a->rank; ++k) {
                    cplx d = alpha * dotu(a->V + k * c, x1, c);
                    const cplx* u = a->U + k * m;
                    for (int64_t i = 0; i < m; ++i) b1[i] += u[i] * d;
                }
            }
            for (int64_t i = 0; i < m; ++i) b[rows[i]] += b1[i];
        }
    free(x1); free(b1);
}

void oc_hmatrix_gemv(const oc_hmatrix* h, const double* alpha, const double* x,
                     const double* beta, double* b) {
    hm_gemv(h, alpha[0] + I * alpha[1], (const cplx*)x, beta[0] + I * beta[1], (cplx*)b);
}

void oc_hmatrix_to_full(const oc_hmatrix* h, double* Ad, int64_t lda) {
    cplx* A = (cplx*)Ad;
    for (int64_t j = 0; j < h->n; ++j)
        for (int64_t i = 0; i < h->n; ++i) A[j * lda + i] = 0;
    for (int64_t blk = 0; blk < h->bl.nblocks; ++blk) {
        const int64_t* rows = h->bl.rows + h->bl.row_off[blk];
        const int64_t* cols = h->bl.cols + h->bl.col_off[blk];
        int64_t m = h->bl.row_off[blk + 1] - h->bl.row_off[blk];
        int64_t c = h->bl.col_off[blk + 1] - h->bl.col_off[blk];
        for (int64_t j = 0; j < c; ++j)
            for (int64_t i = 0; i < m; ++i) {
                cplx v;
                if (h->bl.admissible[blk]) {
                    v = 0;
                    for (int64_t k = 0; k < h->lr[blk].rank; ++k)
                        v += h->lr[blk].U[k * m + i] * h->lr[blk].V[k * c + j];
                } else v = h->dense[blk][j * m + i];
                A[cols[j] * lda + rows[i]] += v;
            }
    }
}

void oc_hmatrix_stats(const oc_hmatrix* h, int64_t* st) {
    st[0] = st[1] = st[2] = st[3] = 0;
    for (int64_t b = 0; b < h->bl.nblocks; ++b) {
        int64_t m = h->bl.row_off[b + 1] - h->bl.row_off[b];
        int64_t c = h->bl.col_off[b + 1] - h->bl.col_off[b];
        if (h->bl.admissible[b]) { st[0]++; st[2] += h->lr[b].rank * (m + c); st[3] += h->lr[b].rank; }
        else { st[1]++; st[2] += m * c; }
    }
}

static void hm_mv(void* c, const cplx* x, cplx* y) {
    const oc_hmatrix* h = (const oc_hmatrix*)c;
    for (int64_t i = 0; i < h->n; ++i) y[i] = 0;
    hm_gemv(h, 1.0, x, 0.0, y);
}

int oc_gmres_hmatrix(const oc_hmatrix* h, int64_t max_it, double tol, double* x, oc_gmres_report* rep) {
    return gmres_generic(h->n, hm_mv, (void*)h, h->norm, max_it, tol, (cplx*)x, rep);
}

/* ======================================================================= */
/* solve.rs:11-185 */
typedef struct { const oc_problem* p; int side; } bem_gen_ctx;
static void bem_gen(void* c, const int64_t* Iv, int64_t ni, const int64_t* Jv, int64_t nj, double* out) {
    const bem_gen_ctx* g = (const bem_gen_ctx*)c;
    oc_row_or_column(g->p, Iv, ni, Jv, nj, g->side, out);
}

static int solve_dense(const oc_problem* p, const cplx* A, int64_t n, cplx* x, oc_gmres_report* rep) {
    if (p->solver == OC_DIRECT) return oc_lu_solve(n, (const double*)A, n, (double*)x);
    return oc_gmres_dense(n, (const double*)A, n, p->max_iterations, p->tolerance, (double*)x, rep);
}

int oc_solve_for_surface(const oc_problem* p, const double* rhs_incd, double* phid, double* vnd,
                         oc_gmres_report* rep, int nthreads) {
    int64_t n = p->n;
    const cplx* rhs_inc = (const cplx*)rhs_incd;
    cplx* phi = (cplx*)phid;
    cplx* vn = (cplx*)vnd;
    if (rep) memset(rep, 0, sizeof *rep);
    for (int64_t i = 0; i < n; ++i) { phi[i] = 0; vn[i] = 0; }
    cplx bcv = p->bc_value[0] + I * p->bc_value[1];
    double omega = omega_of(p);
    if (p->solver != OC_HIERARCHICAL) {
        /* get_surface_dense (solve.rs:24-71) */
        cplx* H = (cplx*)malloc(sizeof(cplx) * (size_t)(n * n));
        cplx* G = (cplx*)malloc(sizeof(cplx) * (size_t)(n * n));
        oc_dense_surface(p, (double*)H, (double*)G, n, nthreads);
        int st = 0;
        if (p->bc_type == OC_BC_PRESSURE) {
            for (int64_t i = 0; i < n; ++i) { phi[i] = bcv; vn[i] = rhs_inc[i]; }
            for (int64_t j = 0; j < n; ++j) {
                cplx f = -1.0 * phi[j];
                for (int64_t i = 0; i < n; ++i) vn[i] += H[j * n + i] * f;
            }
            st = solve_dense(p, G, n, vn, rep);
        } else if (p->bc_type == OC_BC_NORMAL_VELOCITY) {
            for (int64_t i = 0; i < n; ++i) { vn[i] = bcv; phi[i] = -rhs_inc[i]; }
            for (int64_t j = 0; j < n; ++j) {
                cplx f = vn[j];
                for (int64_t i = 0; i < n; ++i) phi[i] += G[j * n + i] * f;
            }
            st = solve_dense(p, H, n, phi, rep);
        } else {
            cplx factor = (-I * (omega * p->mass_density)) / bcv;
            for (int64_t t = 0; t < n * n; ++t) H[t] += factor * G[t];
            for (int64_t i = 0; i < n; ++i) phi[i] = -rhs_inc[i];
            st = solve_dense(p, H, n, phi, rep);
            for (int64_t i = 0; i < n; ++i) vn[i] = factor * phi[i];
        }
        free(H); free(G);
        return st;
    }
    /* get_surface_hmatrix (solve.rs:74-150) */
    cplx* rhs = (cplx*)malloc(sizeof(cplx) * (size_t)n);
    memcpy(rhs, rhs_inc, sizeof(cplx) * (size_t)n);
    int zero_bc = p->bc_value[0] == 0.0 && p->bc_value[1] == 0.0;
    if (p->bc_type == OC_BC_IMPEDANCE) {
        for (int64_t i = 0; i < n; ++i) rhs[i] = -rhs_inc[i];
    } else {
        oc_hmatrix* hr = NULL;
        if (!zero_bc) {
            bem_gen_ctx gc = {p, 0};
            hr = oc_hmatrix_build(n, p->cpts, OC_CPT_STRIDE, p->hm_leaf, p->hm_eta, p->hm_aca_tol, bem_gen, &gc);
            if (!hr) { free(rhs); return 1; }
        }
        cplx* fillv = (cplx*)malloc(sizeof(cplx) * (size_t)n);
        for (int64_t i = 0; i < n; ++i) fillv[i] = bcv;
        cplx bet = (p->bc_type == OC_BC_PRESSURE) ? 1.0 : -1.0;
        if (p->bc_type == OC_BC_PRESSURE) for (int64_t i = 0; i < n; ++i) phi[i] = bcv;
        else for (int64_t i = 0; i < n; ++i) vn[i] = bcv;
        if (hr) hm_gemv(hr, 1.0, fillv, bet, rhs);
        else if (bet != 1.0) for (int64_t i = 0; i < n; ++i) rhs[i] *= bet;
        free(fillv);
        oc_hmatrix_free(hr);
    }
    bem_gen_ctx gl = {p, 1};
    oc_hmatrix* hl = oc_hmatrix_build(n, p->cpts, OC_CPT_STRIDE, p->hm_leaf, p->hm_eta, p->hm_aca_tol, bem_gen, &gl);
    if (!hl) { free(rhs); return 1; }
    int st = oc_gmres_hmatrix(hl, p->max_iterations, p->tolerance, (double*)rhs, rep);
    oc_hmatrix_free(hl);
    if (p->bc_type == OC_BC_PRESSURE) memcpy(vn, rhs, sizeof(cplx) * (size_t)n);
    else if (p->bc_type == OC_BC_NORMAL_VELOCITY) memcpy(phi, rhs, sizeof(cplx) * (size_t)n);
    else {
        memcpy(phi, rhs, sizeof(cplx) * (size_t)n);
        cplx factor = (-I * (omega * p->mass_density)) / bcv;
        for (int64_t i = 0; i < n; ++i) vn[i] = factor * phi[i];
    }
    free(rhs);
    return st;
}

/* solve.rs:173-185: phi_fp = [phi_inc if Total] - M phi + L vn */
void oc_get_field(const oc_problem* p, const double* Md, const double* Ld, int64_t ld,
                  const double* phid, const double* vnd, const double* incd, double* outd) {
    const cplx* M = (const cplx*)Md;
    const cplx* L = (const cplx*)Ld;
    const cplx* phi = (const cplx*)phid;
    const cplx* vn = (const cplx*)vnd;
    const cplx* inc = (const cplx*)incd;
    cplx* out = (cplx*)outd;
    for (int64_t i = 0; i < p->nfp; ++i) out[i] = p->output_total ? inc[i] : 0.0;
    for (int64_t j = 0; j < p->n; ++j) {
        cplx f = -1.0 * phi[j];
        for (int64_t i = 0; i < p->nfp; ++i) out[i] += M[j * ld + i] * f;
    }
    for (int64_t j = 0; j < p->n; ++j) {
        cplx f = vn[j];
        for (int64_t i = 0; i < p->nfp; ++i) out[i] += L[j * ld + i] * f;
    }
}

/* postprocess.rs:83-87: p = (i omega rho) phi */
void oc_convert_to_pressure(const oc_problem* p, double* vd, int64_t n) {
    cplx* v = (cplx*)vd;
    cplx s = I * (omega_of(p) * p->mass_density);
    for (int64_t i = 0; i < n; ++i) v[i] *= s;
}

/* analysis.rs:87-111, one frequency. */
int oc_run_frequency(const oc_problem* p, double* phi, double* vn, double* fps, double* fpi,
                     oc_gmres_report* rep, int nthreads) {
    int64_t n = p->n;
    double* rhs = (double*)malloc(sizeof(double) * 2 * (size_t)n);
    oc_incident_surface(p, rhs);
    int st = oc_solve_for_surface(p, rhs, phi, vn, rep, nthreads);
    free(rhs);
    int64_t nfp = p->nfp;
    if (nfp > 0) {
        double* M = (double*)malloc(sizeof(double) * 2 * (size_t)(nfp * n));
        double* L = (double*)malloc(sizeof(double) * 2 * (size_t)(nfp * n));
        oc_dense_field(p, M, L, nfp);
        oc_incident_field(p, fpi);
        oc_get_field(p, M, L, nfp, phi, vn, fpi, fps);
        free(M); free(L);
    }
    return st;
}
