/*
 * oracle.c -- CPU oracle for the OLDG field step. TEST INFRASTRUCTURE ONLY:
 * it is the checker for the CUDA library (tests/, __graft_entry__.smoke())
 * and the timed CPU baseline (bench.py's cpu_baseline and --impl reference);
 * nothing in the product links or calls it.
 *
 * A plain-C restatement of the reference's algorithm, written to share as
 * little as possible with the CUDA path:
 *   - wide derivative, gradient and Laplacian passes: src/evolution.jl:24-35,
 *     67-110 (wide_derivative, gradient_kernel!, laplacian_kernel!), with the
 *     stencil applied over its full (P+3)-wide window;
 *   - ghosts: each ghost point finds its neighbour by locating the point just
 *     across the face in a finest-level cell map (not by the library's face
 *     table), then applies the documented TreeAMR element-local semantics
 *     (reference CODE.md "The layout", "Reflecting walls", "The coupling"):
 *     injection at equal level, mirror with u even and d_d u odd at walls,
 *     and across coarse-fine faces the coarse element's Lagrange polynomial
 *     evaluated at the fine node (I) or the adjoint restriction
 *     R = M_c^-1 I^T M_f, both evaluated here from the nodes and weights;
 *   - truncation: the dense projector el.truncate applied along each
 *     dimension of each element (the matrix the reference's tests compare
 *     the rank-one kernel against, test/evolution_tests.jl:83-103);
 *   - RK4: the classic tableau, truncation as stage and step limiter
 *     (src/evolution.jl:1408-1430), u^{n+1} = T(u + dt/6 (k1+2k2+2k3+k4));
 *   - energy, norm: src/evolution.jl:1472-1489, src/layout.jl:100-122,223-235;
 *   - modal indicator: src/refinement.jl:56-100, 147-179.
 * Tables (nodes, weights, stencil, projector, duals) come from the caller:
 * the tests load them from tests/golden/element_tables.json, an mpmath
 * 512-bit restatement of src/element.jl.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
    int D, P, E, nblocks, truncate;
    int roots[3], periodic[3], reflecting[3];
    double lo[3], hi[3];
    const int32_t* level;
    const int64_t* corner;
    const double* nodes;     /* P+1 */
    const double* weights;   /* P+1 */
    const double* stencil;   /* (P+1) x (P+3) row-major */
    const double* projector; /* (P+1) x (P+1) row-major */
    const double* duals;     /* (P+1) x (P+1) row-major */
    /* diagonal metric (NULL: flat): node values sqrt(g), A_1..A_D per block,
     * (N^D, 1+D, nblocks) column-major; and the sqrt(g) factor along each
     * element line at its nodes, (P+1, E, nblocks, D), from which the oracle
     * builds the line's orthogonal projector itself */
    const double* coef;
    const double* line_weights;
    /* full metric (metric == 2, D = 3): coef holds sqrt(g), S[d][i] (10 per
     * node); the explicit face table of a glued forest (face_nb, face_code as
     * in the library's descriptor); elem_slot[b] != 0 marks blocks whose
     * truncation is the sqrt(g)-orthogonal projection per element (solved
     * here from the nodes, weights and sqrt(g)); Dirichlet data: the plane wave
     * (wave_k, wave_phi) at the boundary face nodes' positions bnd_x ((3, N^2)
     * per slot); t the time of the state */
    int metric;
    const int32_t* face_nb;
    const int32_t* face_code;
    const int32_t* elem_slot;
    const double* bnd_x;
    double wave_k[3];
    double wave_phi;
    double t;
    /* the boundary faces' condition: 0 the Dirichlet plane wave, 1 radiative
     * (src/evolution.jl:1129-1260): u's ghost is the face node's u, and the
     * face's flux is F* = -sigma |S[d]| (kappa v + inv_r u); 2 the Dirichlet
     * spherical standing wave j0(k r) cos(k t), k = wave_k[0] */
    int boundary;
    double kappa, inv_r;
    /* the per-element projections' LU factors with partial pivoting, built by
     * oracle_full_prepare (NULL: each projection factors its own Gram matrix) */
    void* cache;
    /* a refined brick patch (the ball's affine cube, face_nb -2 between its
     * blocks): built by oracle_full_prepare from the blocks' level and corner
     * in a brick of roots[k] root blocks */
    void* brick;
} oracle_mesh;

typedef struct {
    const oracle_mesh* m;
    int N, P1;
    int64_t NN;       /* nodes per block */
    int lmax;
    int64_t grid[3];  /* finest cells per dim */
    int32_t* owner;   /* finest cell -> leaf */
    double cellw;     /* root block width (physical) */
} ctx_t;

static int64_t ipow64(int64_t b, int e) { int64_t r = 1; while (e-- > 0) r *= b; return r; }

static int ctx_init(ctx_t* c, const oracle_mesh* m) {
    c->m = m;
    c->P1 = m->P + 1;
    c->N = m->E * c->P1;
    c->NN = ipow64(c->N, m->D);
    c->lmax = 0;
    for (int b = 0; b < m->nblocks; ++b) if (m->level[b] > c->lmax) c->lmax = m->level[b];
    int64_t total = 1;
    for (int k = 0; k < 3; ++k) {
        c->grid[k] = k < m->D ? ((int64_t)m->roots[k] << c->lmax) : 1;
        total *= c->grid[k];
    }
    c->owner = (int32_t*)malloc(sizeof(int32_t) * total);
    if (!c->owner) return -1;
    for (int64_t i = 0; i < total; ++i) c->owner[i] = -1;
    for (int b = 0; b < m->nblocks; ++b) {
        int64_t span = (int64_t)1 << (c->lmax - m->level[b]);
        int64_t c0[3] = {0, 0, 0}, c1[3] = {1, 1, 1};
        for (int k = 0; k < m->D; ++k) { c0[k] = m->corner[(int64_t)b * m->D + k] * span; c1[k] = c0[k] + span; }
        for (int64_t z = c0[2]; z < c1[2]; ++z)
            for (int64_t y = c0[1]; y < c1[1]; ++y)
                for (int64_t x = c0[0]; x < c1[0]; ++x)
                    c->owner[x + c->grid[0] * (y + c->grid[1] * z)] = b;
    }
    c->cellw = (m->hi[0] - m->lo[0]) / m->roots[0];
    return 0;
}

/* The leaf containing point x (in root-block units), with periodic wrap;
 * -1 outside a non-periodic domain. */
static int locate(const ctx_t* c, const double* x) {
    int64_t i[3] = {0, 0, 0};
    for (int k = 0; k < c->m->D; ++k) {
        double s = x[k] * (double)((int64_t)1 << c->lmax);
        int64_t v = (int64_t)floor(s);
        if (v < 0 || v >= c->grid[k]) {
            if (!c->m->periodic[k]) return -1;
            v = ((v % c->grid[k]) + c->grid[k]) % c->grid[k];
        }
        i[k] = v;
    }
    return c->owner[i[0] + c->grid[0] * (i[1] + c->grid[1] * i[2])];
}

static double block_width(const ctx_t* c, int b) { return 1.0 / (double)((int64_t)1 << c->m->level[b]); }
static double block_origin(const ctx_t* c, int b, int k) {
    return (double)c->m->corner[(int64_t)b * c->m->D + k] * block_width(c, b);
}
static double spacing(const ctx_t* c, int b) { return c->cellw * block_width(c, b) / c->N; }

static int64_t oidx(const ctx_t* c, const int* x) {
    int64_t r = 0, s = 1;
    for (int k = 0; k < c->m->D; ++k) { r += x[k] * s; s *= c->N; }
    return r;
}

static double lagrange(const double* xi, int n, int j, double x) {
    double r = 1.0;
    for (int k = 0; k < n; ++k) if (k != j) r *= (x - xi[k]) / (xi[j] - xi[k]);
    return r;
}

/* The ghost across face (d, side) of block b at the face node whose
 * tangential owned coordinates are x[k] (k != d), read from the owned field
 * `f` (N^D per block). parity is the wall sign. */
static double ghost_value(const ctx_t* c, int b, int d, int side, const int* x, const double* f, double parity) {
    const oracle_mesh* m = c->m;
    const int D = m->D, P1 = c->P1, N = c->N, E = m->E;
    double w = block_width(c, b);
    double ew = w / E;
    double pt[3];
    for (int k = 0; k < D; ++k) {
        if (k == d) pt[k] = side ? block_origin(c, b, k) + w + 0.25 * ew : block_origin(c, b, k) - 0.25 * ew;
        else pt[k] = block_origin(c, b, k) + ((x[k] / P1) + 0.5) * ew;
    }
    int nb = locate(c, pt);
    if (nb < 0) {
        /* reflecting wall: the mirror of this block's own face node */
        int y[3] = {0, 0, 0};
        for (int k = 0; k < D; ++k) y[k] = k == d ? (side ? N - 1 : 0) : x[k];
        return parity * f[(int64_t)b * c->NN + oidx(c, y)];
    }
    int ln = m->level[nb], lb = m->level[b];
    int y[3] = {0, 0, 0};
    y[d] = side ? 0 : N - 1;
    const double* fn = f + (int64_t)nb * c->NN;
    if (ln == lb) {
        for (int k = 0; k < D; ++k) if (k != d) y[k] = x[k];
        return fn[oidx(c, y)];
    }
    double wn = block_width(c, nb), ewn = wn / E;
    if (ln == lb - 1) {
        /* fine ghost from the coarse neighbour: its element's polynomial at our node */
        int ec[3] = {0, 0, 0};
        double xi[3] = {0, 0, 0};
        for (int k = 0; k < D; ++k) {
            if (k == d) continue;
            int e = x[k] / P1, i = x[k] % P1;
            double center = block_origin(c, b, k) + (e + 0.5) * ew;
            double rel = center - block_origin(c, nb, k);
            /* periodic images never split a tangential coordinate: faces are inside the box tangentially */
            ec[k] = (int)floor(rel / ewn);
            double mid = block_origin(c, nb, k) + (ec[k] + 0.5) * ewn;
            int half = center > mid ? 1 : 0;
            xi[k] = (m->nodes[i] + (half ? 1.0 : -1.0)) / 2.0;
        }
        double acc = 0.0;
        int tk[2], nt = 0;
        for (int k = 0; k < D; ++k) if (k != d) tk[nt++] = k;
        int64_t combos = ipow64(P1, nt);
        for (int64_t q = 0; q < combos; ++q) {
            double wgt = 1.0;
            int64_t qq = q;
            for (int a = 0; a < nt; ++a) {
                int k = tk[a], j = (int)(qq % P1);
                qq /= P1;
                wgt *= lagrange(m->nodes, P1, j, xi[k]);
                y[k] = ec[k] * P1 + j;
            }
            acc += wgt * fn[oidx(c, y)];
        }
        return acc;
    }
    /* coarse ghost from the fine neighbours: R = M_c^-1 I^T M_f over the
     * 2(P+1) fine nodes of our element along each tangential dimension */
    {
        int tk[2], nt = 0;
        for (int k = 0; k < D; ++k) if (k != d) tk[nt++] = k;
        int ecur[3] = {0, 0, 0}, jn[3] = {0, 0, 0};
        for (int a = 0; a < nt; ++a) { int k = tk[a]; ecur[k] = x[k] / P1; jn[k] = x[k] % P1; }
        int64_t combos = ipow64(2 * P1, nt);
        double acc = 0.0;
        for (int64_t q = 0; q < combos; ++q) {
            double wgt = 1.0;
            double ptf[3];
            int rr[3] = {0, 0, 0}, half[3] = {0, 0, 0};
            int64_t qq = q;
            for (int a = 0; a < nt; ++a) {
                int k = tk[a];
                int r = (int)(qq % (2 * P1));
                qq /= 2 * P1;
                rr[k] = r % P1;
                half[k] = r / P1;
                double xc = (m->nodes[rr[k]] + (half[k] ? 1.0 : -1.0)) / 2.0;
                wgt *= lagrange(m->nodes, P1, jn[k], xc) * m->weights[rr[k]] / (2.0 * m->weights[jn[k]]);
                ptf[k] = block_origin(c, b, k) + (ecur[k] + 0.25 + 0.5 * half[k]) * ew;
            }
            ptf[d] = pt[d];
            int fb = locate(c, ptf);
            if (fb < 0) return NAN;
            int z[3] = {0, 0, 0};
            z[d] = side ? 0 : N - 1;
            for (int a = 0; a < nt; ++a) {
                int k = tk[a];
                double rel = ptf[k] - block_origin(c, fb, k);
                int fe = (int)floor(rel / (block_width(c, fb) / E));
                z[k] = fe * P1 + rr[k];
            }
            acc += wgt * f[(int64_t)fb * c->NN + oidx(c, z)];
        }
        return acc;
    }
}

/* D_d a / h at every owned node of block b, with a's ghosts across the two
 * faces normal to d (src/evolution.jl:24-35). */
static void derivative_block(const ctx_t* c, int b, int d, const double* a, double parity, double* out,
                             const double* scale) {
    const oracle_mesh* m = c->m;
    const int N = c->N, P1 = c->P1, PW = m->P + 3;
    const double h = spacing(c, b);
    const double* ab = a + (int64_t)b * c->NN;
    int x[3] = {0, 0, 0};
    for (int64_t n = 0; n < c->NN; ++n) {
        int64_t r = n;
        for (int k = 0; k < m->D; ++k) { x[k] = (int)(r % N); r /= N; }
        int I = x[d];
        int i = I % P1;
        int start = I - i - 1;
        double acc = 0.0;
        for (int k = 0; k < PW; ++k) {
            int pos = start + k;
            double val;
            if (pos < 0 || pos >= N) {
                double coef = m->stencil[i * PW + k];
                if (coef == 0.0) continue;
                val = ghost_value(c, b, d, pos >= N, x, a, parity);
            } else {
                int y[3] = {x[0], x[1], x[2]};
                y[d] = pos;
                val = ab[oidx(c, y)];
            }
            acc += m->stencil[i * PW + k] * val;
        }
        out[n] = acc / h;
        if (scale) out[n] *= scale[n];
    }
}

int oracle_rhs(const oracle_mesh* m, const double* u, double* du) {
    ctx_t c;
    if (ctx_init(&c, m)) return -1;
    const int D = m->D;
    const int64_t NN = c.NN, nb = m->nblocks;
    double* ua = (double*)malloc(sizeof(double) * NN * nb);
    double* g = (double*)malloc(sizeof(double) * NN * nb * D);
    if (!ua || !g) { free(ua); free(g); free(c.owner); return -1; }
#pragma omp parallel for schedule(dynamic)
    for (int64_t b = 0; b < nb; ++b) memcpy(ua + b * NN, u + b * 2 * NN, sizeof(double) * NN);
#pragma omp parallel for schedule(dynamic)
    for (int64_t b = 0; b < nb; ++b)
        for (int d = 0; d < D; ++d)
            derivative_block(&c, (int)b, d, ua, 1.0, g + (int64_t)d * NN * nb + b * NN,
                             m->coef ? m->coef + (b * (1 + D) + 1 + d) * NN : NULL);
#pragma omp parallel
    {
        double* tmp = (double*)malloc(sizeof(double) * NN);
#pragma omp for schedule(dynamic)
        for (int64_t b = 0; b < nb; ++b) {
            double* dv = du + b * 2 * NN + NN;
            for (int64_t n = 0; n < NN; ++n) dv[n] = 0.0;
            for (int d = 0; d < D; ++d) {
                derivative_block(&c, (int)b, d, g + (int64_t)d * NN * nb, -1.0, tmp, NULL);
                for (int64_t n = 0; n < NN; ++n) dv[n] += tmp[n];
            }
            /* on a geometry: sqrt(g) v' = sum_d D_d F_d */
            if (m->coef)
                for (int64_t n = 0; n < NN; ++n) dv[n] /= m->coef[b * (1 + D) * NN + n];
            memcpy(du + b * 2 * NN, u + b * 2 * NN + NN, sizeof(double) * NN);
        }
        free(tmp);
    }
    free(ua);
    free(g);
    free(c.owner);
    return 0;
}

/* The reference's Laplacian divides the summed second derivatives by h once,
 * with each gradient already divided by h: D_d(D_d u / h) / h. The routine
 * above divides both passes' stencil sums by h, which is the same value. */

/* The line's projector onto degree < P orthogonal in sum_i w_i a_i f_i g_i:
 * Pi = I - phi (x) dual with phi = L_P less its projection on L_0..L_{P-1},
 * dual = w a phi / gamma (src/evolution.jl:578-622), in long double. */
static void line_projector(const oracle_mesh* m, const double* a, double* Pi) {
    const int P = m->P, P1 = P + 1;
    long double L[16][16], G[16][17], phi[16], c[16];
    for (int i = 0; i < P1; ++i) {
        long double x = m->nodes[i];
        L[0][i] = 1.0L;
        if (P >= 1) L[1][i] = x;
        for (int k = 2; k <= P; ++k) L[k][i] = ((2 * k - 1) * x * L[k - 1][i] - (k - 1) * L[k - 2][i]) / k;
    }
    for (int k = 0; k < P; ++k) {
        for (int l = 0; l < P; ++l) {
            long double s = 0;
            for (int i = 0; i < P1; ++i) s += (long double)m->weights[i] * a[i] * L[k][i] * L[l][i];
            G[k][l] = s;
        }
        long double r = 0;
        for (int i = 0; i < P1; ++i) r += (long double)m->weights[i] * a[i] * L[P][i] * L[k][i];
        G[k][P] = r;
    }
    for (int k = 0; k < P; ++k) { /* Gaussian elimination with partial pivoting */
        int piv = k;
        for (int r = k + 1; r < P; ++r) if (fabsl(G[r][k]) > fabsl(G[piv][k])) piv = r;
        for (int j = 0; j <= P; ++j) { long double t = G[k][j]; G[k][j] = G[piv][j]; G[piv][j] = t; }
        for (int r = k + 1; r < P; ++r) {
            long double f = G[r][k] / G[k][k];
            for (int j = k; j <= P; ++j) G[r][j] -= f * G[k][j];
        }
    }
    for (int k = P - 1; k >= 0; --k) {
        long double s = G[k][P];
        for (int j = k + 1; j < P; ++j) s -= G[k][j] * c[j];
        c[k] = s / G[k][k];
    }
    long double gamma = 0;
    for (int i = 0; i < P1; ++i) {
        long double v = L[P][i];
        for (int k = 0; k < P; ++k) v -= c[k] * L[k][i];
        phi[i] = v;
        gamma += (long double)m->weights[i] * a[i] * v * v;
    }
    for (int i = 0; i < P1; ++i)
        for (int j = 0; j < P1; ++j)
            Pi[i * P1 + j] = (double)((i == j ? 1.0L : 0.0L) - phi[i] * m->weights[j] * a[j] * phi[j] / gamma);
}

static void truncate_with(const ctx_t* c, double* u) {
    const oracle_mesh* m = c->m;
    const int D = m->D, N = c->N, P1 = c->P1, E = m->E;
    const int64_t NN = c->NN;
    const int64_t nel = ipow64(E, D);
#pragma omp parallel for schedule(dynamic)
    for (int64_t b = 0; b < m->nblocks; ++b) {
        double* v = u + b * 2 * NN + NN;
        double line[16], out[16];
        for (int64_t el = 0; el < nel; ++el) {
            int base[3] = {0, 0, 0};
            int64_t r = el;
            for (int k = 0; k < D; ++k) { base[k] = (int)(r % E) * P1; r /= E; }
            for (int d = 0; d < D; ++d) {
                int64_t nl = ipow64(P1, D - 1);
                double Pline[256];
                const double* Pm = m->projector;
                if (m->line_weights) {
                    /* the line's own projector: element index along d is base[d] / P1 */
                    const double* a = m->line_weights + (int64_t)P1 * (base[d] / P1 + (int64_t)E * (b + (int64_t)m->nblocks * d));
                    line_projector(m, a, Pline);
                    Pm = Pline;
                }
                for (int64_t l = 0; l < nl; ++l) {
                    int x[3] = {base[0], base[1], base[2]};
                    int64_t ll = l;
                    for (int k = 0; k < D; ++k) if (k != d) { x[k] += (int)(ll % P1); ll /= P1; }
                    for (int j = 0; j < P1; ++j) { int y[3] = {x[0], x[1], x[2]}; y[d] += j; line[j] = v[oidx(c, y)]; }
                    for (int i = 0; i < P1; ++i) {
                        double s = 0.0;
                        for (int j = 0; j < P1; ++j) s += Pm[i * P1 + j] * line[j];
                        out[i] = s;
                    }
                    for (int i = 0; i < P1; ++i) { int y[3] = {x[0], x[1], x[2]}; y[d] += i; v[oidx(c, y)] = out[i]; }
                }
            }
        }
    }
    (void)N;
}

int oracle_truncate(const oracle_mesh* m, double* u) {
    if (!m->truncate) return 0;
    ctx_t c;
    c.m = m;
    c.P1 = m->P + 1;
    c.N = m->E * c.P1;
    c.NN = ipow64(c.N, m->D);
    truncate_with(&c, u);
    return 0;
}

int oracle_rk4(const oracle_mesh* m, double* u, double dt, int nsteps) {
    ctx_t c;
    c.m = m;
    c.P1 = m->P + 1;
    c.N = m->E * c.P1;
    c.NN = ipow64(c.N, m->D);
    const int64_t W = 2 * c.NN * m->nblocks;
    double* k1 = (double*)malloc(sizeof(double) * W);
    double* k2 = (double*)malloc(sizeof(double) * W);
    double* k3 = (double*)malloc(sizeof(double) * W);
    double* k4 = (double*)malloc(sizeof(double) * W);
    double* y = (double*)malloc(sizeof(double) * W);
    if (!k1 || !k2 || !k3 || !k4 || !y) { free(k1); free(k2); free(k3); free(k4); free(y); return -1; }
    int rc = 0;
    for (int s = 0; s < nsteps && rc == 0; ++s) {
        rc |= oracle_rhs(m, u, k1);
#pragma omp parallel for
        for (int64_t i = 0; i < W; ++i) y[i] = u[i] + dt / 2 * k1[i];
        if (m->truncate) truncate_with(&c, y);
        rc |= oracle_rhs(m, y, k2);
#pragma omp parallel for
        for (int64_t i = 0; i < W; ++i) y[i] = u[i] + dt / 2 * k2[i];
        if (m->truncate) truncate_with(&c, y);
        rc |= oracle_rhs(m, y, k3);
#pragma omp parallel for
        for (int64_t i = 0; i < W; ++i) y[i] = u[i] + dt * k3[i];
        if (m->truncate) truncate_with(&c, y);
        rc |= oracle_rhs(m, y, k4);
#pragma omp parallel for
        for (int64_t i = 0; i < W; ++i) u[i] = u[i] + dt / 6 * (k1[i] + 2 * k2[i] + 2 * k3[i] + k4[i]);
        if (m->truncate) truncate_with(&c, u);
    }
    free(k1); free(k2); free(k3); free(k4); free(y);
    return rc;
}

static double node_weight(const ctx_t* c, int b, int64_t n) {
    const oracle_mesh* m = c->m;
    double h = spacing(c, b), w = 1.0;
    for (int k = 0; k < m->D; ++k) { w *= h * c->P1 / 2.0 * m->weights[(n % c->N) % c->P1]; n /= c->N; }
    return w;
}

/* 1/2 sum w (v^2 + sum_d (D_d u)^2), summed block by block in order. */
int oracle_energy(const oracle_mesh* m, const double* u, double* out) {
    ctx_t c;
    if (ctx_init(&c, m)) return -1;
    const int D = m->D;
    const int64_t NN = c.NN, nb = m->nblocks;
    double* ua = (double*)malloc(sizeof(double) * NN * nb);
    double* part = (double*)calloc(nb, sizeof(double));
    if (!ua || !part) { free(ua); free(part); free(c.owner); return -1; }
    for (int64_t b = 0; b < nb; ++b) memcpy(ua + b * NN, u + b * 2 * NN, sizeof(double) * NN);
#pragma omp parallel
    {
        double* g = (double*)malloc(sizeof(double) * NN);
#pragma omp for schedule(dynamic)
        for (int64_t b = 0; b < nb; ++b) {
            double s = 0.0;
            const double* v = u + b * 2 * NN + NN;
            const double* cf = m->coef ? m->coef + b * (1 + D) * NN : NULL;
            for (int64_t n = 0; n < NN; ++n) s += (cf ? cf[n] : 1.0) * node_weight(&c, (int)b, n) * v[n] * v[n];
            for (int d = 0; d < D; ++d) {
                /* on a geometry the flux F_d = A_d D_d u enters as F_d^2 / A_d */
                derivative_block(&c, (int)b, d, ua, 1.0, g, cf ? cf + (1 + d) * NN : NULL);
                for (int64_t n = 0; n < NN; ++n)
                    s += node_weight(&c, (int)b, n) * g[n] * g[n] / (cf ? cf[(1 + d) * NN + n] : 1.0);
            }
            part[b] = 0.5 * s;
        }
        free(g);
    }
    double e = 0.0;
    for (int64_t b = 0; b < nb; ++b) e += part[b];
    *out = e;
    free(ua);
    free(part);
    free(c.owner);
    return 0;
}

/* Volume-normalised p-norm of u - ref (ref may be NULL); p = 0: largest |value|. */
int oracle_norm(const oracle_mesh* m, const double* u, const double* ref, int p, int vars_mask, double* out) {
    ctx_t c;
    c.m = m;
    c.P1 = m->P + 1;
    c.N = m->E * c.P1;
    c.NN = ipow64(c.N, m->D);
    c.cellw = (m->hi[0] - m->lo[0]) / m->roots[0];
    double num = 0.0, vol = 0.0;
    for (int64_t b = 0; b < m->nblocks; ++b)
        for (int var = 0; var < 2; ++var) {
            if (!(vars_mask & (1 << var))) continue;
            for (int64_t n = 0; n < c.NN; ++n) {
                int64_t o = b * 2 * c.NN + var * c.NN + n;
                double x = fabs(u[o] - (ref ? ref[o] : 0.0));
                double w = node_weight(&c, (int)b, n);
                if (m->coef) w *= m->coef[b * (1 + m->D) * c.NN + n];
                if (p == 0) num = x > num ? x : num;
                else num += w * pow(x, p);
                vol += w;
            }
        }
    *out = p == 0 ? num : (vol == 0 ? 0.0 : pow(num / vol, 1.0 / p));
    return 0;
}

/* tau per element: post * max over lines in every dim and modes q of
 * (weights[q] |sum_j duals[modes[q]][j] a_j| / peak)^pows[q]. */
int oracle_modes(const oracle_mesh* m, const double* u, int var, int nq, const int* modes, const double* weights,
                 const double* pows, double post, double* tau) {
    const int D = m->D, P1 = m->P + 1, E = m->E, N = E * P1;
    const int64_t NN = ipow64(N, D), nel = ipow64(E, D);
    double peak = 0.0;
    for (int64_t b = 0; b < m->nblocks; ++b)
        for (int64_t n = 0; n < NN; ++n) {
            double x = fabs(u[b * 2 * NN + (int64_t)var * NN + n]);
            peak = x > peak ? x : peak;
        }
    double scale = peak == 0.0 ? 0.0 : 1.0 / peak;
    for (int64_t b = 0; b < m->nblocks; ++b) {
        const double* a = u + b * 2 * NN + (int64_t)var * NN;
        for (int64_t el = 0; el < nel; ++el) {
            int base[3] = {0, 0, 0};
            int64_t r = el;
            for (int k = 0; k < D; ++k) { base[k] = (int)(r % E) * P1; r /= E; }
            double best = 0.0;
            for (int d = 0; d < D; ++d) {
                int64_t nl = ipow64(P1, D - 1);
                for (int64_t l = 0; l < nl; ++l) {
                    int x[3] = {base[0], base[1], base[2]};
                    int64_t ll = l;
                    for (int k = 0; k < D; ++k) if (k != d) { x[k] += (int)(ll % P1); ll /= P1; }
                    for (int q = 0; q < nq; ++q) {
                        double cq = 0.0;
                        for (int j = 0; j < P1; ++j) {
                            int y[3] = {x[0], x[1], x[2]};
                            y[d] += j;
                            int64_t o = 0, s = 1;
                            for (int k = 0; k < D; ++k) { o += y[k] * s; s *= N; }
                            cq += m->duals[modes[q] * P1 + j] * a[o];
                        }
                        double v = pow(weights[q] * scale * fabs(cq), pows[q]);
                        best = v > best ? v : best;
                    }
                }
            }
            tau[b * nel + el] = post * best;
        }
    }
    return 0;
}

int oracle_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}


/* ------------------------------------------------------------------------- */
/* The full metric (src/evolution.jl:112-220, 266-425, 1110-1127).           */

static int oriented_t(int t, int N, int code) {
    int a = t % N, b = t / N;
    if (code & 1) { int s = a; a = b; b = s; }
    if (code & 2) a = N - 1 - a;
    if (code & 4) b = N - 1 - b;
    return a + N * b;
}

/* Owned coordinates of face f's node at tangential t (other dims in
 * increasing order, first fastest) with x_d = xd. */
static void face_node(int N, int f, int t, int xd, int* x) {
    int d = f / 2, k2 = 0;
    int tt[2] = {t % N, t / N};
    for (int k = 0; k < 3; ++k) x[k] = k == d ? xd : tt[k2++];
}

/* The spherical standing wave u = j0(k r) cos(k t), j0(x) = sin(x)/x, an
 * exact solution of the wave equation regular at the origin, and its
 * Cartesian gradient k j0'(k r) cos(k t) x / r, j0'(x) = (x cos x - sin x)/x^2:
 * the Dirichlet data of boundary kind 2 (k = wave_k[0]), the stand-in for any
 * data(x, t) of the reference's DirichletValues (src/evolution.jl:1110-1127). */
static double standing_u(const oracle_mesh* m, const double* X, int F, int t, double time, double* grad) {
    const double k = m->wave_k[0];
    const double x = X[t], y = X[F + t], z = X[2 * F + t];
    const double r = sqrt(x * x + y * y + z * z), kr = k * r, c = cos(k * time);
    const double j0 = kr > 1e-6 ? sin(kr) / kr : 1 - kr * kr / 6;
    const double dj0 = kr > 1e-6 ? (kr * cos(kr) - sin(kr)) / (kr * kr) : -kr / 3;
    if (grad) {
        const double g = r > 0 ? k * dj0 * c / r : 0.0;
        grad[0] = g * x;
        grad[1] = g * y;
        grad[2] = g * z;
    }
    return j0 * c;
}

static double wave_phase(const oracle_mesh* m, const double* X, int F, int t, double time) {
    double om = sqrt(m->wave_k[0] * m->wave_k[0] + m->wave_k[1] * m->wave_k[1] + m->wave_k[2] * m->wave_k[2]);
    return m->wave_k[0] * X[t] + m->wave_k[1] * X[F + t] + m->wave_k[2] * X[2 * F + t] - om * time + m->wave_phi;
}

/* The ghost of field `f` (ncomp components of N^3 per block, component
 * stride `cs`) across face `face` of block b at tangential t: the
 * neighbour's face node, oriented; or NAN for a boundary face. */
static double full_ghost(const oracle_mesh* m, int N, int64_t NN, const double* f, int64_t bstride, int comp,
                         int64_t cs, int b, int face, int t) {
    int nb = m->face_nb[b * 6 + face];
    if (nb < 0) return NAN;
    int code = m->face_code[b * 6 + face];
    int nf = code & 15, o = (code >> 4) & 7;
    int t2 = oriented_t(t, N, o);
    int x[3];
    face_node(N, nf, t2, (nf & 1) ? N - 1 : 0, x);
    (void)NN;
    return f[nb * bstride + comp * cs + x[0] + N * (x[1] + N * x[2])];
}

/* A refined brick patch inside the ball (its affine cube): its blocks as a
 * forest of their own, whose ghosts across the faces between them are the
 * flat problem's (ghost_value: injection, or the coarse element's polynomial
 * at a fine node, or the restriction R = M_c^-1 I^T M_f), located in its own
 * finest-cell map; `f` holds one field over the brick's blocks. */
typedef struct {
    oracle_mesh sub;
    ctx_t ctx;
    int nb;
    int* local;        /* global block -> brick block, or -1 */
    int* global;       /* brick block -> global block */
    int32_t* level;
    int64_t* corner;
    double* f;         /* one field over the brick's blocks, N^3 each */
} brick_t;

static void brick_free(brick_t* br) {
    if (!br) return;
    free(br->local); free(br->global); free(br->level); free(br->corner); free(br->f); free(br->ctx.owner);
    free(br);
}

static brick_t* brick_build(const oracle_mesh* m) {
    const int N = m->E * (m->P + 1);
    const int64_t NN = (int64_t)N * N * N;
    int nb = 0;
    for (int b = 0; b < m->nblocks; ++b)
        for (int f = 0; f < 6; ++f)
            if (m->face_nb[b * 6 + f] == -2) { ++nb; break; }
    if (nb == 0) return NULL;
    brick_t* br = (brick_t*)calloc(1, sizeof(brick_t));
    br->local = (int*)malloc(sizeof(int) * m->nblocks);
    br->global = (int*)malloc(sizeof(int) * nb);
    br->level = (int32_t*)malloc(sizeof(int32_t) * nb);
    br->corner = (int64_t*)malloc(sizeof(int64_t) * 3 * nb);
    br->f = (double*)malloc(sizeof(double) * NN * nb);
    br->nb = nb;
    int k = 0;
    for (int b = 0; b < m->nblocks; ++b) {
        br->local[b] = -1;
        for (int f = 0; f < 6; ++f)
            if (m->face_nb[b * 6 + f] == -2) {
                br->local[b] = k;
                br->global[k] = b;
                br->level[k] = m->level[b];
                for (int q = 0; q < 3; ++q) br->corner[3 * k + q] = m->corner[(int64_t)b * 3 + q];
                ++k;
                break;
            }
    }
    br->sub = *m;
    br->sub.nblocks = nb;
    br->sub.level = br->level;
    br->sub.corner = br->corner;
    for (int q = 0; q < 3; ++q) {
        br->sub.periodic[q] = 0;
        br->sub.reflecting[q] = 1;
        br->sub.lo[q] = 0.0;
        br->sub.hi[q] = (double)m->roots[q];
    }
    br->sub.cache = NULL;
    br->sub.brick = NULL;
    if (ctx_init(&br->ctx, &br->sub)) { brick_free(br); return NULL; }
    return br;
}

/* Copy component `comp` of a field (bstride words per block, component
 * stride cs) of the brick's blocks into br->f. */
static void brick_gather(brick_t* br, const double* fld, int64_t NN, int64_t bstride, int comp, int64_t cs) {
    for (int l = 0; l < br->nb; ++l)
        memcpy(br->f + (int64_t)l * NN, fld + (int64_t)br->global[l] * bstride + comp * cs, sizeof(double) * NN);
}

/* The logical node spacing of block b: a root block spans 1, a level-L block 2^-L. */
static double full_spacing(const oracle_mesh* m, int b, int N) {
    return 1.0 / N / (double)((int64_t)1 << m->level[b]);
}

/* V = grad u at every node of every block, (3, N^3) per block. */
static void full_gradient(const oracle_mesh* m, const double* u, double* V) {
    const int P = m->P, P1 = P + 1, PW = P + 3, N = m->E * P1;
    const int64_t NN = (int64_t)N * N * N, F = (int64_t)N * N;
    brick_t* br = (brick_t*)m->brick;
    if (br) brick_gather(br, u, NN, 2 * NN, 0, 0);
#pragma omp parallel for schedule(dynamic)
    for (int b = 0; b < m->nblocks; ++b) {
        const double* cf = m->coef + (int64_t)b * 10 * NN;
        const double h = full_spacing(m, b, N);
        for (int64_t n = 0; n < NN; ++n) {
            int x[3] = {(int)(n % N), (int)((n / N) % N), (int)(n / F)};
            double De[3];
            for (int e = 0; e < 3; ++e) {
                int i = x[e] % P1, start = x[e] - i - 1;
                double acc = 0;
                for (int k = 0; k < PW; ++k) {
                    double coefk = m->stencil[i * PW + k];
                    if (coefk == 0.0) continue;
                    int pos = start + k;
                    double val;
                    if (pos < 0 || pos >= N) {
                        int face = 2 * e + (pos >= N), t = 0, k2 = 0;
                        int tt[2];
                        for (int q = 0; q < 3; ++q) if (q != e) tt[k2++] = x[q];
                        t = tt[0] + N * tt[1];
                        if (m->face_nb[b * 6 + face] == -2) {
                            val = ghost_value(&br->ctx, br->local[b], e, pos >= N, x, br->f, 1.0);
                            acc += coefk * val;
                            continue;
                        }
                        val = full_ghost(m, N, NN, u, 2 * NN, 0, 0, b, face, t);
                        if (isnan(val) && m->boundary == 1) {
                            int y[3] = {x[0], x[1], x[2]};
                            y[e] = pos < 0 ? 0 : N - 1;
                            val = u[(int64_t)b * 2 * NN + y[0] + N * (y[1] + N * y[2])];
                        } else if (isnan(val) && m->boundary == 2) {
                            const double* X = m->bnd_x + ((int64_t)b * 6 + face) * 3 * F;
                            val = standing_u(m, X, (int)F, t, m->t, NULL);
                        } else if (isnan(val)) {
                            const double* X = m->bnd_x + ((int64_t)b * 6 + face) * 3 * F;
                            val = sin(wave_phase(m, X, (int)F, t, m->t));
                        }
                    } else {
                        int y[3] = {x[0], x[1], x[2]};
                        y[e] = pos;
                        val = u[(int64_t)b * 2 * NN + y[0] + N * (y[1] + N * y[2])];
                    }
                    acc += coefk * val;
                }
                De[e] = acc / h;
            }
            for (int ci = 0; ci < 3; ++ci) {
                double s = 0;
                for (int e = 0; e < 3; ++e) s += cf[(1 + 3 * e + ci) * NN + n] * De[e];
                V[(int64_t)b * 3 * NN + ci * NN + n] = s / cf[n];
            }
        }
    }
}

int oracle_rhs_full(const oracle_mesh* m, const double* u, double* du) {
    const int P = m->P, P1 = P + 1, PW = P + 3, N = m->E * P1;
    const int64_t NN = (int64_t)N * N * N, F = (int64_t)N * N;
    double* V = (double*)malloc(sizeof(double) * 3 * NN * m->nblocks);
    if (!V) return -1;
    full_gradient(m, u, V);
    /* the brick's V components, each a field of its own for ghost_value */
    brick_t* br = (brick_t*)m->brick;
    double* Vb[3] = {NULL, NULL, NULL};
    if (br) {
        for (int ci = 0; ci < 3; ++ci) {
            Vb[ci] = (double*)malloc(sizeof(double) * NN * br->nb);
            if (!Vb[ci]) { for (int q = 0; q < 3; ++q) free(Vb[q]); free(V); return -1; }
            for (int l = 0; l < br->nb; ++l)
                memcpy(Vb[ci] + (int64_t)l * NN, V + (int64_t)br->global[l] * 3 * NN + ci * NN, sizeof(double) * NN);
        }
    }
#pragma omp parallel for schedule(dynamic)
    for (int b = 0; b < m->nblocks; ++b) {
        const double* cf = m->coef + (int64_t)b * 10 * NN;
        const double h = full_spacing(m, b, N);
        for (int64_t n = 0; n < NN; ++n) {
            int x[3] = {(int)(n % N), (int)((n / N) % N), (int)(n / F)};
            double lap = 0;
            for (int d = 0; d < 3; ++d) {
                int i = x[d] % P1, start = x[d] - i - 1;
                double acc = 0;
                for (int k = 0; k < PW; ++k) {
                    double coefk = m->stencil[i * PW + k];
                    if (coefk == 0.0) continue;
                    int pos = start + k;
                    int y[3] = {x[0], x[1], x[2]};
                    double Vw[3];
                    int64_t sn;                      /* the node whose S[d] forms the flux */
                    if (pos < 0 || pos >= N) {
                        int face = 2 * d + (pos >= N), k2 = 0, tt[2];
                        for (int q = 0; q < 3; ++q) if (q != d) tt[k2++] = x[q];
                        int t = tt[0] + N * tt[1];
                        y[d] = pos < 0 ? 0 : N - 1;
                        sn = y[0] + N * (y[1] + N * y[2]);
                        if (m->face_nb[b * 6 + face] == -2) {
                            for (int ci = 0; ci < 3; ++ci)
                                Vw[ci] = ghost_value(&br->ctx, br->local[b], d, pos >= N, x, Vb[ci], 1.0);
                            double Fd = 0;
                            for (int ci = 0; ci < 3; ++ci) Fd += cf[(1 + 3 * d + ci) * NN + sn] * Vw[ci];
                            acc += coefk * Fd;
                            continue;
                        }
                        if (m->face_nb[b * 6 + face] < 0 && m->boundary == 1) {
                            /* the ghost's flux 2 F* - F: the central flux is F* */
                            double Fo = 0, S2 = 0;
                            for (int ci = 0; ci < 3; ++ci) {
                                double Sc = cf[(1 + 3 * d + ci) * NN + sn];
                                Fo += Sc * V[(int64_t)b * 3 * NN + ci * NN + sn];
                                S2 += Sc * Sc;
                            }
                            double sigma = pos >= N ? 1.0 : -1.0;
                            double us = u[(int64_t)b * 2 * NN + sn], vs = u[(int64_t)b * 2 * NN + NN + sn];
                            double Fstar = -sigma * sqrt(S2) * (m->kappa * vs + m->inv_r * us);
                            acc += coefk * (2 * Fstar - Fo);
                            continue;
                        }
                        if (m->face_nb[b * 6 + face] < 0 && m->boundary == 2) {
                            const double* X = m->bnd_x + ((int64_t)b * 6 + face) * 3 * F;
                            standing_u(m, X, (int)F, t, m->t, Vw);
                        } else if (m->face_nb[b * 6 + face] < 0) {
                            const double* X = m->bnd_x + ((int64_t)b * 6 + face) * 3 * F;
                            double c = cos(wave_phase(m, X, (int)F, t, m->t));
                            for (int ci = 0; ci < 3; ++ci) Vw[ci] = m->wave_k[ci] * c;
                        } else {
                            for (int ci = 0; ci < 3; ++ci)
                                Vw[ci] = full_ghost(m, N, NN, V, 3 * NN, ci, NN, b, face, t);
                        }
                    } else {
                        y[d] = pos;
                        sn = y[0] + N * (y[1] + N * y[2]);
                        for (int ci = 0; ci < 3; ++ci) Vw[ci] = V[(int64_t)b * 3 * NN + ci * NN + sn];
                    }
                    double Fd = 0;
                    for (int ci = 0; ci < 3; ++ci) Fd += cf[(1 + 3 * d + ci) * NN + sn] * Vw[ci];
                    acc += coefk * Fd;
                }
                lap += acc / h;
            }
            du[(int64_t)b * 2 * NN + n] = u[(int64_t)b * 2 * NN + NN + n];
            du[(int64_t)b * 2 * NN + NN + n] = lap / cf[n];
        }
    }
    free(V);
    for (int ci = 0; ci < 3; ++ci) free(Vb[ci]);
    return 0;
}

/* Legendre L_q at the nodes, q <= P, in long double. */
static void legendre_nodes(const oracle_mesh* m, long double L[16][16]) {
    const int P = m->P, P1 = P + 1;
    for (int i = 0; i < P1; ++i) {
        long double x = m->nodes[i];
        L[0][i] = 1.0L;
        if (P >= 1) L[1][i] = x;
        for (int k = 2; k <= P; ++k) L[k][i] = ((2 * k - 1) * x * L[k - 1][i] - (k - 1) * L[k - 2][i]) / k;
    }
}

/* The Gram matrix Psi^T W Psi of one element (m3 x m3, row stride m3 + 1),
 * its weights W and node indices. */
static void element_gram(const oracle_mesh* m, const double* cf, int N, const int* base, long double L[16][16],
                         long double* Gm, long double* W, int64_t* idx) {
    const int P = m->P, P1 = P + 1, n3 = P1 * P1 * P1, m3 = P * P * P;
    for (int nn = 0; nn < n3; ++nn) {
        int n0 = nn % P1, n1 = (nn / P1) % P1, n2 = nn / (P1 * P1);
        idx[nn] = (base[0] + n0) + (int64_t)N * ((base[1] + n1) + (int64_t)N * (base[2] + n2));
        W[nn] = (long double)m->weights[n0] * m->weights[n1] * m->weights[n2] * cf[idx[nn]];
    }
    for (int q = 0; q < m3; ++q) {
        int q0 = q % P, q1 = (q / P) % P, q2 = q / (P * P);
        for (int r = 0; r < m3; ++r) {
            int r0 = r % P, r1 = (r / P) % P, r2 = r / (P * P);
            long double s = 0;
            for (int nn = 0; nn < n3; ++nn) {
                int n0 = nn % P1, n1 = (nn / P1) % P1, n2 = nn / (P1 * P1);
                s += L[q0][n0] * L[q1][n1] * L[q2][n2] * W[nn] * L[r0][n0] * L[r1][n1] * L[r2][n2];
            }
            Gm[q * (m3 + 1) + r] = s;
        }
    }
}

/* Gaussian elimination with partial pivoting of the m3 x m3 part of Gm (row
 * stride m3 + 1), in place: the multipliers below the diagonal, the row
 * swaps in piv. */
static void lu_factor(long double* Gm, int m3, int* piv) {
#define G(i, j) Gm[(i) * (m3 + 1) + (j)]
    for (int k = 0; k < m3; ++k) {
        int p = k;
        for (int r = k + 1; r < m3; ++r) if (fabsl(G(r, k)) > fabsl(G(p, k))) p = r;
        piv[k] = p;
        if (p != k)
            for (int j = 0; j < m3; ++j) { long double t = G(k, j); G(k, j) = G(p, j); G(p, j) = t; }
        for (int r = k + 1; r < m3; ++r) {
            long double f = G(r, k) / G(k, k);
            G(r, k) = f;
            for (int j = k + 1; j < m3; ++j) G(r, j) -= f * G(k, j);
        }
    }
#undef G
}

/* v <- Psi z with (Psi^T W Psi) z = Psi^T W v, through the LU factors. */
static void lu_project(const oracle_mesh* m, const long double* Gm, const int* piv, const long double* W,
                       const int64_t* idx, long double L[16][16], double* v) {
    const int P = m->P, P1 = P + 1, n3 = P1 * P1 * P1, m3 = P * P * P;
#define G(i, j) Gm[(i) * (m3 + 1) + (j)]
    long double z[729];
    for (int q = 0; q < m3; ++q) {
        int q0 = q % P, q1 = (q / P) % P, q2 = q / (P * P);
        long double c = 0;
        for (int nn = 0; nn < n3; ++nn) {
            int n0 = nn % P1, n1 = (nn / P1) % P1, n2 = nn / (P1 * P1);
            c += L[q0][n0] * L[q1][n1] * L[q2][n2] * W[nn] * v[idx[nn]];
        }
        z[q] = c;
    }
    for (int k = 0; k < m3; ++k) {
        if (piv[k] != k) { long double t = z[k]; z[k] = z[piv[k]]; z[piv[k]] = t; }
        for (int r = k + 1; r < m3; ++r) z[r] -= G(r, k) * z[k];
    }
    for (int k = m3 - 1; k >= 0; --k) {
        long double s = z[k];
        for (int j = k + 1; j < m3; ++j) s -= G(k, j) * z[j];
        z[k] = s / G(k, k);
    }
#undef G
    for (int nn = 0; nn < n3; ++nn) {
        int n0 = nn % P1, n1 = (nn / P1) % P1, n2 = nn / (P1 * P1);
        long double s = 0;
        for (int q = 0; q < m3; ++q) {
            int q0 = q % P, q1 = (q / P) % P, q2 = q / (P * P);
            s += L[q0][n0] * L[q1][n1] * L[q2][n2] * z[q];
        }
        v[idx[nn]] = (double)s;
    }
}

/* Per projected element (blocks in order, elements e0 fastest): the LU
 * factors and pivots, the weights and node indices. */
typedef struct {
    int nelem;
    int64_t* first;      /* per block: its first element's index, or -1 */
    long double* lu;     /* m3 (m3 + 1) per element */
    int* piv;            /* m3 per element */
    long double* w;      /* n3 per element */
    int64_t* idx;        /* n3 per element */
} proj_cache_t;

/* The sqrt(g)-orthogonal projection onto Q_{P-1} of one element's v:
 * solve (Psi^T W Psi) z = Psi^T W v, v = Psi z, in long double. */
static void full_project_element(const oracle_mesh* m, const double* cf, double* v, int N, const int* base) {
    const int P = m->P, m3 = P * P * P;
    long double L[16][16];
    legendre_nodes(m, L);
    long double* Gm = (long double*)malloc(sizeof(long double) * m3 * (m3 + 1));
    int* piv = (int*)malloc(sizeof(int) * m3);
    if (!Gm || !piv) { free(Gm); free(piv); return; }
    long double W[1000];
    int64_t idx[1000];
    element_gram(m, cf, N, base, L, Gm, W, idx);
    lu_factor(Gm, m3, piv);
    lu_project(m, Gm, piv, W, idx, L, v);
    free(Gm);
    free(piv);
}

int oracle_full_prepare(oracle_mesh* m) {
    const int P = m->P, P1 = P + 1, E = m->E, N = E * P1;
    const int n3 = P1 * P1 * P1, m3 = P * P * P, EE = E * E * E;
    const int64_t NN = (int64_t)N * N * N;
    proj_cache_t* c = (proj_cache_t*)calloc(1, sizeof(proj_cache_t));
    if (!c) return -1;
    c->first = (int64_t*)malloc(sizeof(int64_t) * m->nblocks);
    int nel = 0;
    for (int b = 0; b < m->nblocks; ++b) {
        c->first[b] = m->elem_slot[b] ? nel : -1;
        if (m->elem_slot[b]) nel += EE;
    }
    c->nelem = nel;
    c->lu = (long double*)malloc(sizeof(long double) * (size_t)nel * m3 * (m3 + 1) + 1);
    c->piv = (int*)malloc(sizeof(int) * (size_t)nel * m3 + 1);
    c->w = (long double*)malloc(sizeof(long double) * (size_t)nel * n3 + 1);
    c->idx = (int64_t*)malloc(sizeof(int64_t) * (size_t)nel * n3 + 1);
    if (!c->first || !c->lu || !c->piv || !c->w || !c->idx) {
        free(c->first); free(c->lu); free(c->piv); free(c->w); free(c->idx); free(c);
        return -1;
    }
    long double L[16][16];
    legendre_nodes(m, L);
#pragma omp parallel for schedule(dynamic)
    for (int b = 0; b < m->nblocks; ++b) {
        if (c->first[b] < 0) continue;
        const double* cf = m->coef + (int64_t)b * 10 * NN;
        for (int e = 0; e < EE; ++e) {
            const int64_t k = c->first[b] + e;
            int base[3] = {(e % E) * P1, ((e / E) % E) * P1, (e / (E * E)) * P1};
            long double* Gm = c->lu + k * m3 * (m3 + 1);
            element_gram(m, cf, N, base, L, Gm, c->w + k * n3, c->idx + k * n3);
            lu_factor(Gm, m3, c->piv + k * m3);
        }
    }
    m->cache = c;
    m->brick = brick_build(m);
    return 0;
}

void oracle_full_release(oracle_mesh* m) {
    brick_free((brick_t*)m->brick);
    m->brick = NULL;
    proj_cache_t* c = (proj_cache_t*)m->cache;
    if (!c) return;
    free(c->first); free(c->lu); free(c->piv); free(c->w); free(c->idx); free(c);
    m->cache = NULL;
}

/* The tensor projector on the affine blocks and the element projection on
 * the others, from the state before truncation (`orig`). */
static void full_truncate_from(const oracle_mesh* m, const double* orig, double* u) {
    const int P1 = m->P + 1, E = m->E, N = E * P1;
    const int64_t NN = (int64_t)N * N * N;
    ctx_t c;
    c.m = m;
    c.P1 = P1;
    c.N = N;
    c.NN = NN;
    memcpy(u, orig, sizeof(double) * 2 * NN * m->nblocks);
    truncate_with(&c, u);
    const proj_cache_t* pc = (const proj_cache_t*)m->cache;
    const int P = m->P, m3 = P * P * P, n3 = P1 * P1 * P1;
#pragma omp parallel for schedule(dynamic)
    for (int b = 0; b < m->nblocks; ++b) {
        if (!m->elem_slot[b]) continue;
        double* v = u + (int64_t)b * 2 * NN + NN;
        memcpy(v, orig + (int64_t)b * 2 * NN + NN, sizeof(double) * NN);
        const double* cf = m->coef + (int64_t)b * 10 * NN;
        long double L[16][16];
        legendre_nodes(m, L);
        for (int e2 = 0; e2 < E; ++e2)
            for (int e1 = 0; e1 < E; ++e1)
                for (int e0 = 0; e0 < E; ++e0) {
                    int base[3] = {e0 * P1, e1 * P1, e2 * P1};
                    if (pc) {
                        const int64_t k = pc->first[b] + e0 + E * (e1 + E * e2);
                        lu_project(m, pc->lu + k * m3 * (m3 + 1), pc->piv + k * m3, pc->w + k * n3,
                                   pc->idx + k * n3, L, v);
                    } else {
                        full_project_element(m, cf, v, N, base);
                    }
                }
    }
}

int oracle_truncate_full2(const oracle_mesh* m, double* u) {
    if (!m->truncate) return 0;
    const int64_t W = 2 * (int64_t)m->E * (m->P + 1) * m->E * (m->P + 1) * m->E * (m->P + 1) * m->nblocks;
    double* orig = (double*)malloc(sizeof(double) * W);
    if (!orig) return -1;
    memcpy(orig, u, sizeof(double) * W);
    full_truncate_from(m, orig, u);
    free(orig);
    return 0;
}

int oracle_rk4_full(oracle_mesh* m, double* u, double t0, double dt, int nsteps) {
    const int64_t NN = (int64_t)m->E * (m->P + 1) * m->E * (m->P + 1) * m->E * (m->P + 1);
    const int64_t W = 2 * NN * m->nblocks;
    double* k1 = (double*)malloc(sizeof(double) * W);
    double* k2 = (double*)malloc(sizeof(double) * W);
    double* k3 = (double*)malloc(sizeof(double) * W);
    double* k4 = (double*)malloc(sizeof(double) * W);
    double* y = (double*)malloc(sizeof(double) * W);
    if (!k1 || !k2 || !k3 || !k4 || !y) { free(k1); free(k2); free(k3); free(k4); free(y); return -1; }
    int rc = 0;
    for (int s = 0; s < nsteps && rc == 0; ++s) {
        const double t = t0 + s * dt;
        m->t = t;
        rc |= oracle_rhs_full(m, u, k1);
        for (int64_t i = 0; i < W; ++i) y[i] = u[i] + dt / 2 * k1[i];
        rc |= oracle_truncate_full2(m, y);
        m->t = t + dt / 2;
        rc |= oracle_rhs_full(m, y, k2);
        for (int64_t i = 0; i < W; ++i) y[i] = u[i] + dt / 2 * k2[i];
        rc |= oracle_truncate_full2(m, y);
        rc |= oracle_rhs_full(m, y, k3);
        for (int64_t i = 0; i < W; ++i) y[i] = u[i] + dt * k3[i];
        rc |= oracle_truncate_full2(m, y);
        m->t = t + dt;
        rc |= oracle_rhs_full(m, y, k4);
        for (int64_t i = 0; i < W; ++i) u[i] = u[i] + dt / 6 * (k1[i] + 2 * k2[i] + 2 * k3[i] + k4[i]);
        rc |= oracle_truncate_full2(m, u);
    }
    free(k1); free(k2); free(k3); free(k4); free(y);
    return rc;
}

/* 1/2 sum w sqrt(g) (v^2 + |V|^2), block by block in order. */
int oracle_energy_full(const oracle_mesh* m, const double* u, double* out) {
    const int P1 = m->P + 1, N = m->E * P1;
    const int64_t NN = (int64_t)N * N * N;
    double* V = (double*)malloc(sizeof(double) * 3 * NN * m->nblocks);
    if (!V) return -1;
    full_gradient(m, u, V);
    double e = 0;
    for (int b = 0; b < m->nblocks; ++b) {
        const double* cf = m->coef + (int64_t)b * 10 * NN;
        const double h = full_spacing(m, b, N);
        double s = 0;
        for (int64_t n = 0; n < NN; ++n) {
            double w = 1;
            int64_t r = n;
            for (int k = 0; k < 3; ++k) { w *= h * P1 / 2.0 * m->weights[(r % N) % P1]; r /= N; }
            double vv = u[(int64_t)b * 2 * NN + NN + n];
            double q = vv * vv;
            for (int ci = 0; ci < 3; ++ci) q += V[(int64_t)b * 3 * NN + ci * NN + n] * V[(int64_t)b * 3 * NN + ci * NN + n];
            s += w * cf[n] * q;
        }
        /* a radiative boundary's own energy: inv_r sum w |S[d]| u^2 over its faces' nodes */
        if (m->boundary == 1 && m->inv_r != 0) {
            for (int face = 0; face < 6; ++face) {
                if (m->face_nb[b * 6 + face] != -1) continue;
                int d = face / 2;
                for (int t = 0; t < N * N; ++t) {
                    int x[3];
                    face_node(N, face, t, (face & 1) ? N - 1 : 0, x);
                    int64_t n = x[0] + (int64_t)N * (x[1] + (int64_t)N * x[2]);
                    double w = 1, S2 = 0;
                    for (int q = 0; q < 3; ++q) if (q != d) w *= h * P1 / 2.0 * m->weights[x[q] % P1];
                    for (int ci = 0; ci < 3; ++ci) S2 += cf[(1 + 3 * d + ci) * NN + n] * cf[(1 + 3 * d + ci) * NN + n];
                    double uu = u[(int64_t)b * 2 * NN + n];
                    s += w * sqrt(S2) * m->inv_r * uu * uu;
                }
            }
        }
        e += 0.5 * s;
    }
    *out = e;
    free(V);
    return 0;
}

/* sqrt(g)-weighted p-norm of u - ref (p = 0: largest |value|). */
int oracle_norm_full(const oracle_mesh* m, const double* u, const double* ref, int p, int vars_mask, double* out) {
    const int P1 = m->P + 1, N = m->E * P1;
    const int64_t NN = (int64_t)N * N * N;
    double num = 0, vol = 0;
    for (int b = 0; b < m->nblocks; ++b)
        for (int var = 0; var < 2; ++var) {
            const double h = full_spacing(m, b, N);
            if (!(vars_mask & (1 << var))) continue;
            for (int64_t n = 0; n < NN; ++n) {
                int64_t o = (int64_t)b * 2 * NN + var * NN + n;
                double x = fabs(u[o] - (ref ? ref[o] : 0.0));
                double w = m->coef[(int64_t)b * 10 * NN + n];
                int64_t r = n;
                for (int k = 0; k < 3; ++k) { w *= h * P1 / 2.0 * m->weights[(r % N) % P1]; r /= N; }
                if (p == 0) num = x > num ? x : num;
                else num += w * pow(x, p);
                vol += w;
            }
        }
    *out = p == 0 ? num : (vol == 0 ? 0.0 : pow(num / vol, 1.0 / p));
    return 0;
}
