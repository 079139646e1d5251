/*
 * refcpu.c -- the reference's threaded CPU field step restated in C, for the
 * timed CPU baseline. TEST INFRASTRUCTURE ONLY: bench.py's cpu_baseline leg
 * and its --impl reference arm time it, and tests/ hold it to the oracle
 * (oracle.c); nothing in the product links or calls it.
 *
 * oracle.c is the independent checker (per-point windows, ghosts located
 * geometrically, dense projectors) and is slow by design. This file instead
 * follows the data flow the reference's package runs on a multicore host,
 * so that its time stands for the reference's CPU path:
 *   - wave_rhs! (src/evolution.jl:1318-1371): u scattered into a working
 *     array with one ghost layer (scatter_u_kernel!, :41-46); its face ghosts
 *     filled by injection of the face neighbour's face-adjacent plane, a
 *     reflecting wall mirroring u even (fill_ghosts!, :1303-1314); the
 *     gradient pass writing D_d u / h into the d-th gradient set, whose ghost
 *     plane is along d only (gradient_kernel!, :67-90); those ghosts filled, a
 *     wall mirroring d_d u odd; the Laplacian pass (laplacian_kernel!,
 *     :92-110). The wide derivative (:24-35) reads the (P+3)-point window of
 *     its element along d. Each pass is a parallel loop over blocks, and the
 *     loops run along element lines, the x lines vectorised across x;
 *   - truncate_state! (:222-264, 1383-1395): per element, dimension by
 *     dimension in the fixed order 1..D, a dot product with topdual and a
 *     rank-one update with topmode;
 *   - the integrator (src/stepping.jl:72-78): classic RK4 with the truncation
 *     as stage and step limiter (:1408-1430), its stage values and update
 *     fused broadcasts over the state, parallel over blocks.
 * OpenMP over blocks with a static schedule; every array is first touched by
 * the thread that later works on it, as the reference's launches by block
 * owner place it. The forest is a uniform brick of root blocks (periodic or
 * reflecting per dimension), which covers every brick the baseline times.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MAXP1 9
#define MAXPW (MAXP1 + 2)

typedef struct {
    int D, P, E, nblocks, truncate;
    int roots[3], reflecting[3];
    const int64_t* corner;   /* nblocks x D level-0 corners */
    double h;                /* node spacing */
    const double* stencil;   /* (P+1) x (P+3) row-major: the wide derivative's rows */
    const double* topmode;   /* P+1 */
    const double* topdual;   /* P+1 */
} refcpu_desc;

typedef struct {
    refcpu_desc d;
    int N, W;                /* nodes per block and dimension; N + 2 */
    int64_t NN;              /* nodes per block */
    int64_t WN;              /* working array per block: (N+2)^D */
    int64_t GN;              /* each gradient set per block: (N+2) N^(D-1) */
    int64_t ws[3];           /* working array strides */
    int64_t gs[3][3];        /* gradient set d's strides */
    int n[3];                /* owned extent per dimension (1 past D) */
    int32_t* nb;             /* nblocks x 2D: the face neighbour, -1 at a wall */
    double* work;
    double* grads[3];
    double* k[4];
    double* y;
    double st[MAXP1 * MAXPW];
    double tm[MAXP1], td[MAXP1];
} refcpu;

int refcpu_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void refcpu_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* first touch by the thread of the block's static share */
static double* alloc_blocks(int nblocks, int64_t per) {
    double* a = (double*)malloc(sizeof(double) * (size_t)nblocks * (size_t)per);
    if (!a) return NULL;
#pragma omp parallel for schedule(static)
    for (int b = 0; b < nblocks; ++b) memset(a + (int64_t)b * per, 0, sizeof(double) * (size_t)per);
    return a;
}

void refcpu_destroy(refcpu* r) {
    if (!r) return;
    free(r->nb);
    free(r->work);
    for (int d = 0; d < 3; ++d) free(r->grads[d]);
    for (int s = 0; s < 4; ++s) free(r->k[s]);
    free(r->y);
    free(r);
}

refcpu* refcpu_create(const refcpu_desc* d) {
    if (d->D < 1 || d->D > 3 || d->P < 1 || d->P + 1 > MAXP1 || d->E < 1 || d->nblocks < 1) return NULL;
    refcpu* r = (refcpu*)calloc(1, sizeof(refcpu));
    if (!r) return NULL;
    r->d = *d;
    const int D = d->D, P1 = d->P + 1, PW = d->P + 3;
    r->N = d->E * P1;
    r->W = r->N + 2;
    r->NN = 1;
    r->WN = 1;
    for (int k = 0; k < D; ++k) { r->NN *= r->N; r->WN *= r->W; }
    r->GN = r->NN / r->N * r->W;
    for (int k = 0; k < 3; ++k) r->n[k] = k < D ? r->N : 1;
    int64_t s = 1;
    for (int k = 0; k < 3; ++k) { r->ws[k] = k < D ? s : 0; if (k < D) s *= r->W; }
    for (int g = 0; g < D; ++g) {
        s = 1;
        for (int k = 0; k < 3; ++k) {
            r->gs[g][k] = k < D ? s : 0;
            if (k < D) s *= (k == g ? r->W : r->N);
        }
    }
    memcpy(r->st, d->stencil, sizeof(double) * P1 * PW);
    memcpy(r->tm, d->topmode, sizeof(double) * P1);
    memcpy(r->td, d->topdual, sizeof(double) * P1);
    /* face neighbours of the uniform brick, found from the level-0 corners */
    int64_t ncell = 1;
    for (int k = 0; k < D; ++k) ncell *= d->roots[k];
    int32_t* at = (int32_t*)malloc(sizeof(int32_t) * ncell);
    r->nb = (int32_t*)malloc(sizeof(int32_t) * (size_t)d->nblocks * 2 * D);
    if (!at || !r->nb) { free(at); refcpu_destroy(r); return NULL; }
    for (int64_t i = 0; i < ncell; ++i) at[i] = -1;
    for (int b = 0; b < d->nblocks; ++b) {
        int64_t key = 0, mul = 1;
        for (int k = 0; k < D; ++k) { key += d->corner[(int64_t)b * D + k] * mul; mul *= d->roots[k]; }
        at[key] = b;
    }
    for (int b = 0; b < d->nblocks; ++b)
        for (int f = 0; f < 2 * D; ++f) {
            const int dd = f / 2, side = f % 2;
            int64_t c[3] = {0, 0, 0};
            for (int k = 0; k < D; ++k) c[k] = d->corner[(int64_t)b * D + k];
            c[dd] += side ? 1 : -1;
            int32_t nbv;
            if (c[dd] < 0 || c[dd] >= d->roots[dd]) {
                if (d->reflecting[dd]) nbv = -1;
                else { c[dd] = (c[dd] + d->roots[dd]) % d->roots[dd]; nbv = -2; }
            } else nbv = -2;
            if (nbv == -2) {
                int64_t key = 0, mul = 1;
                for (int k = 0; k < D; ++k) { key += c[k] * mul; mul *= d->roots[k]; }
                nbv = at[key];
            }
            r->nb[(int64_t)b * 2 * D + f] = nbv;
        }
    free(at);
    r->work = alloc_blocks(d->nblocks, r->WN);
    for (int g = 0; g < D; ++g) r->grads[g] = alloc_blocks(d->nblocks, r->GN);
    for (int q = 0; q < 4; ++q) r->k[q] = alloc_blocks(d->nblocks, 2 * r->NN);
    r->y = alloc_blocks(d->nblocks, 2 * r->NN);
    int ok = r->work && r->y;
    for (int g = 0; g < D; ++g) ok = ok && r->grads[g];
    for (int q = 0; q < 4; ++q) ok = ok && r->k[q];
    if (!ok) { refcpu_destroy(r); return NULL; }
    return r;
}

/* ---- the passes, compiled per order (P1, PW constants) ----------------- */

#define INLINE static inline __attribute__((always_inline))

/* the stored offset of an owned position (x, i1, i2) in the working array */
INLINE int64_t woff(const refcpu* r, int x, int i1, int i2) {
    return (x + 1) + (r->d.D > 1 ? (i1 + 1) * r->ws[1] : 0) + (r->d.D > 2 ? (i2 + 1) * r->ws[2] : 0);
}

/* scatter_u_kernel!: u's owned nodes into the working array */
static void scatter_u(refcpu* r, const double* u) {
    const int N = r->N;
#pragma omp parallel for schedule(static)
    for (int b = 0; b < r->d.nblocks; ++b) {
        const double* ub = u + (int64_t)b * 2 * r->NN;
        double* wb = r->work + (int64_t)b * r->WN;
        for (int i2 = 0; i2 < r->n[2]; ++i2)
            for (int i1 = 0; i1 < r->n[1]; ++i1)
                memcpy(wb + woff(r, 0, i1, i2), ub + (int64_t)N * (i1 + (int64_t)N * i2), sizeof(double) * N);
    }
}

/* fill_ghosts! of u: every face ghost plane of the working array from the
 * face neighbour's face-adjacent owned plane, or the block's own face plane
 * at a reflecting wall (u even) */
static void exchange_u(refcpu* r) {
    const int D = r->d.D, N = r->N;
#pragma omp parallel for schedule(static)
    for (int b = 0; b < r->d.nblocks; ++b) {
        double* wb = r->work + (int64_t)b * r->WN;
        for (int f = 0; f < 2 * D; ++f) {
            const int dd = f / 2, side = f % 2;
            const int32_t nbv = r->nb[(int64_t)b * 2 * D + f];
            const double* src = nbv >= 0 ? r->work + (int64_t)nbv * r->WN : wb;
            /* stored index along dd of the ghost plane and of its source */
            const int gi = side ? N + 1 : 0;
            const int si = nbv >= 0 ? (side ? 1 : N) : (side ? N : 1);
            int t0 = -1, t1 = -1;   /* tangential dims, over their owned range */
            for (int k = 0; k < D; ++k)
                if (k != dd) { if (t0 < 0) t0 = k; else t1 = k; }
            const int n0 = t0 >= 0 ? N : 1, n1 = t1 >= 0 ? N : 1;
            for (int q = 0; q < n1; ++q)
                for (int p = 0; p < n0; ++p) {
                    int64_t o = 0;
                    if (t0 >= 0) o += (int64_t)(p + 1) * r->ws[t0];
                    if (t1 >= 0) o += (int64_t)(q + 1) * r->ws[t1];
                    wb[o + (int64_t)gi * r->ws[dd]] = src[o + (int64_t)si * r->ws[dd]];
                }
        }
    }
}

/* gradient_kernel!: grads[d] (owned + e_d) = D_d u / h */
INLINE void gradient_pass(refcpu* r, const int P1) {
    const int PW = P1 + 2, D = r->d.D, N = r->N, E = r->d.E;
    const double invh = 1.0 / r->d.h;
    const double* st = r->st;
#pragma omp parallel for schedule(static)
    for (int b = 0; b < r->d.nblocks; ++b) {
        const double* wb = r->work + (int64_t)b * r->WN;
        double acc[N];
        /* along x: each x line, element by element */
        {
            double* gb = r->grads[0] + (int64_t)b * r->GN;
            for (int i2 = 0; i2 < r->n[2]; ++i2)
                for (int i1 = 0; i1 < r->n[1]; ++i1) {
                    const double* src = wb + woff(r, 0, i1, i2) - 1;   /* stored x = 0 */
                    double* dst = gb + (int64_t)i1 * r->gs[0][1] + (int64_t)i2 * r->gs[0][2];
                    for (int e = 0; e < E; ++e)
                        for (int i = 0; i < P1; ++i) {
                            double s = 0;
                            for (int k = 0; k < PW; ++k) s += st[i * PW + k] * src[e * P1 + k];
                            dst[e * P1 + i + 1] = s * invh;
                        }
                }
        }
        /* along y and z: each x line of the target, the window's lines summed across x */
        for (int dd = 1; dd < D; ++dd) {
            double* gb = r->grads[dd] + (int64_t)b * r->GN;
            const int64_t sd = r->ws[dd];
            const int other = dd == 1 ? 2 : 1;
            for (int io = 0; io < r->n[other]; ++io)
                for (int I = 0; I < N; ++I) {
                    const int e = I / P1, i = I % P1;
                    const double* row = st + i * PW;
                    int i1 = dd == 1 ? I : io, i2 = dd == 1 ? io : I;
                    /* the window's first stored line along dd: element start - 1 */
                    const double* src = wb + woff(r, 0, i1, i2) + (int64_t)(e * P1 - I - 1) * sd;
                    for (int x = 0; x < N; ++x) acc[x] = 0;
                    for (int k = 0; k < PW; ++k) {
                        const double c = row[k];
                        const double* s = src + (int64_t)k * sd;
                        for (int x = 0; x < N; ++x) acc[x] += c * s[x];
                    }
                    double* dst = gb + (int64_t)(dd == 1 ? I + 1 : i1) * r->gs[dd][1] +
                                  (int64_t)(dd == 2 ? I + 1 : i2) * r->gs[dd][2];
                    for (int x = 0; x < N; ++x) dst[x] = acc[x] * invh;
                }
        }
    }
}

/* fill_ghosts! of the gradient sets: the ghost planes along d from the face
 * neighbour's face-adjacent plane, or the block's own face plane negated at a
 * reflecting wall (d_d u odd) */
static void exchange_grads(refcpu* r) {
    const int D = r->d.D, N = r->N;
#pragma omp parallel for schedule(static)
    for (int b = 0; b < r->d.nblocks; ++b)
        for (int dd = 0; dd < D; ++dd) {
            double* gb = r->grads[dd] + (int64_t)b * r->GN;
            const int64_t* gs = r->gs[dd];
            for (int side = 0; side < 2; ++side) {
                const int32_t nbv = r->nb[(int64_t)b * 2 * D + 2 * dd + side];
                const double* src = nbv >= 0 ? r->grads[dd] + (int64_t)nbv * r->GN : gb;
                const double sign = nbv >= 0 ? 1.0 : -1.0;
                const int gi = side ? N + 1 : 0;
                const int si = nbv >= 0 ? (side ? 1 : N) : (side ? N : 1);
                int t0 = -1, t1 = -1;   /* tangential dims */
                for (int k = 0; k < D; ++k)
                    if (k != dd) { if (t0 < 0) t0 = k; else t1 = k; }
                const int n0 = t0 >= 0 ? N : 1, n1 = t1 >= 0 ? N : 1;
                for (int q = 0; q < n1; ++q)
                    for (int p = 0; p < n0; ++p) {
                        int64_t o = 0;
                        if (t0 >= 0) o += (int64_t)p * gs[t0];
                        if (t1 >= 0) o += (int64_t)q * gs[t1];
                        gb[o + (int64_t)gi * gs[dd]] = sign * src[o + (int64_t)si * gs[dd]];
                    }
            }
        }
}

/* laplacian_kernel!: du = (v, sum_d D_d grads[d] / h) */
INLINE void laplacian_pass(refcpu* r, const double* u, double* du, const int P1) {
    const int PW = P1 + 2, D = r->d.D, N = r->N, E = r->d.E;
    const double invh = 1.0 / r->d.h;
    const double* st = r->st;
#pragma omp parallel for schedule(static)
    for (int b = 0; b < r->d.nblocks; ++b) {
        const double* ub = u + (int64_t)b * 2 * r->NN;
        double* dub = du + (int64_t)b * 2 * r->NN;
        memcpy(dub, ub + r->NN, sizeof(double) * r->NN);
        double t[3][N];
        for (int i2 = 0; i2 < r->n[2]; ++i2)
            for (int i1 = 0; i1 < r->n[1]; ++i1) {
                /* x term along the line */
                const double* g0 = r->grads[0] + (int64_t)b * r->GN + (int64_t)i1 * r->gs[0][1] +
                                   (int64_t)i2 * r->gs[0][2];
                for (int e = 0; e < E; ++e)
                    for (int i = 0; i < P1; ++i) {
                        double s = 0;
                        for (int k = 0; k < PW; ++k) s += st[i * PW + k] * g0[e * P1 + k];
                        t[0][e * P1 + i] = s;
                    }
                for (int dd = 1; dd < D; ++dd) {
                    const int I = dd == 1 ? i1 : i2;
                    const int e = I / P1, i = I % P1;
                    const double* row = st + i * PW;
                    const int64_t sd = r->gs[dd][dd];
                    /* stored index along dd of the window's start: e P1 */
                    const double* src = r->grads[dd] + (int64_t)b * r->GN + (int64_t)(e * P1) * sd +
                                        (dd == 1 ? (int64_t)i2 * r->gs[1][2] : (int64_t)i1 * r->gs[2][1]);
                    for (int x = 0; x < N; ++x) t[dd][x] = 0;
                    for (int k = 0; k < PW; ++k) {
                        const double c = row[k];
                        const double* s = src + (int64_t)k * sd;
                        for (int x = 0; x < N; ++x) t[dd][x] += c * s[x];
                    }
                }
                double* out = dub + r->NN + (int64_t)N * (i1 + (int64_t)N * i2);
                for (int x = 0; x < N; ++x) {
                    double a = t[0][x];
                    if (D > 1) a += t[1][x];
                    if (D > 2) a += t[2][x];
                    out[x] = a * invh;
                }
            }
    }
}

/* truncate_kernel!: v of every element, dimension by dimension */
INLINE void truncate_v(refcpu* r, double* u, const int P1) {
    if (!r->d.truncate) return;
    const int D = r->d.D, N = r->N, E = r->d.E;
    const double* tm = r->tm;
    const double* td = r->td;
#pragma omp parallel for schedule(static)
    for (int b = 0; b < r->d.nblocks; ++b) {
        double* a = u + (int64_t)b * 2 * r->NN + r->NN;
        double c[N];
        /* d = x: each x line, element by element */
        for (int64_t line = 0; line < r->NN / N; ++line) {
            double* l = a + line * N;
            for (int e = 0; e < E; ++e) {
                double s = 0;
                for (int j = 0; j < P1; ++j) s += td[j] * l[e * P1 + j];
                for (int i = 0; i < P1; ++i) l[e * P1 + i] -= tm[i] * s;
            }
        }
        /* d = y, z: lines along d, all x at once */
        for (int dd = 1; dd < D; ++dd) {
            const int64_t sd = dd == 1 ? N : (int64_t)N * N;
            const int other = D == 3 ? (dd == 1 ? 2 : 1) : -1;
            const int no = other >= 0 ? N : 1;
            const int64_t so = other == 2 ? (int64_t)N * N : N;
            for (int io = 0; io < no; ++io)
                for (int e = 0; e < E; ++e) {
                    double* base = a + (other >= 0 ? (int64_t)io * so : 0) + (int64_t)(e * P1) * sd;
                    for (int x = 0; x < N; ++x) c[x] = 0;
                    for (int j = 0; j < P1; ++j)
                        for (int x = 0; x < N; ++x) c[x] += td[j] * base[(int64_t)j * sd + x];
                    for (int i = 0; i < P1; ++i)
                        for (int x = 0; x < N; ++x) base[(int64_t)i * sd + x] -= tm[i] * c[x];
                }
        }
    }
}

INLINE void rhs_impl(refcpu* r, const double* u, double* du, const int P1) {
    scatter_u(r, u);
    exchange_u(r);
    gradient_pass(r, P1);
    exchange_grads(r);
    laplacian_pass(r, u, du, P1);
}

/* y = u + a k, over the whole state */
static void axpy(const refcpu* r, double* restrict y, const double* restrict u, double a,
                 const double* restrict k) {
    const int64_t per = 2 * r->NN;
#pragma omp parallel for schedule(static)
    for (int b = 0; b < r->d.nblocks; ++b) {
        const int64_t o = (int64_t)b * per;
        for (int64_t i = 0; i < per; ++i) y[o + i] = u[o + i] + a * k[o + i];
    }
}

INLINE void rk4_impl(refcpu* r, double* u, double dt, int nsteps, const int P1) {
    const int64_t per = 2 * r->NN;
    for (int n = 0; n < nsteps; ++n) {
        rhs_impl(r, u, r->k[0], P1);
        axpy(r, r->y, u, 0.5 * dt, r->k[0]);
        truncate_v(r, r->y, P1);
        rhs_impl(r, r->y, r->k[1], P1);
        axpy(r, r->y, u, 0.5 * dt, r->k[1]);
        truncate_v(r, r->y, P1);
        rhs_impl(r, r->y, r->k[2], P1);
        axpy(r, r->y, u, dt, r->k[2]);
        truncate_v(r, r->y, P1);
        rhs_impl(r, r->y, r->k[3], P1);
        const double dt6 = dt / 6;
        const double* restrict k1 = r->k[0];
        const double* restrict k2 = r->k[1];
        const double* restrict k3 = r->k[2];
        const double* restrict k4 = r->k[3];
#pragma omp parallel for schedule(static)
        for (int b = 0; b < r->d.nblocks; ++b) {
            const int64_t o = (int64_t)b * per;
            for (int64_t i = o; i < o + per; ++i) u[i] = u[i] + dt6 * (k1[i] + 2 * k2[i] + 2 * k3[i] + k4[i]);
        }
        truncate_v(r, u, P1);
    }
}

#define DISPATCH(call)                                   \
    switch (r->d.P + 1) {                                \
        case 2: call(2); break;                          \
        case 3: call(3); break;                          \
        case 4: call(4); break;                          \
        case 5: call(5); break;                          \
        case 6: call(6); break;                          \
        case 7: call(7); break;                          \
        case 8: call(8); break;                          \
        case 9: call(9); break;                          \
        default: break;                                  \
    }

void refcpu_rhs(refcpu* r, const double* u, double* du) {
#define CALL(p1) rhs_impl(r, u, du, p1)
    DISPATCH(CALL)
#undef CALL
}

void refcpu_truncate(refcpu* r, double* u) {
#define CALL(p1) truncate_v(r, u, p1)
    DISPATCH(CALL)
#undef CALL
}

void refcpu_rk4(refcpu* r, double* u, double dt, int nsteps) {
#define CALL(p1) rk4_impl(r, u, dt, nsteps, p1)
    DISPATCH(CALL)
#undef CALL
}
