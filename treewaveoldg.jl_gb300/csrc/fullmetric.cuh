// The full-metric field step (3D): a geometry whose glues may swap axes,
// such as the seven- and thirteen-patch balls (src/evolution.jl:112-220,
// 266-425, 1110-1299). The gradient crosses faces as Cartesian components
// V = grad u, so a stage is two passes:
//   fm_gradient_kernel: the logical derivatives D_e u at every node (u's face
//     ghosts from the neighbours' exported face nodes, oriented across the
//     glue, the Dirichlet data, or the radiative face's own node), then the
//     fluxes F^d = S[d] . V = sum_e M^de D_e u / h with M^de = S[d] . S[e] /
//     sqrt(g) = sqrt(g) g^de, three words per node, and V = sum_e S[e] D_e u /
//     (h sqrt(g)) only on the face planes, for the neighbours;
//   fm_stage_kernel: sqrt(g) v' = sum_d D_d F^d with the ghost's flux formed
//     from the neighbour's V with this face node's own S[d] (or the Dirichlet
//     gradient, or the radiative 2F* - F); then the RK combination, the
//     sqrt(g)-orthogonal truncation of v per element (Cholesky solves, the
//     factored projection, or the element's tensor projector on an affine
//     patch) and u's face export.
// coef holds, per block, (N^3, 10): sqrt(g), then S[d][i] at 1 + 3d + i; M
// (N^3, 6): M^00, M^11, M^22, M^01, M^02, M^12, formed by the host from coef.
#pragma once

#include "kernels.cuh"
#include "stage3r.cuh"

namespace twoldg {

// Boundary data: the plane wave u = sin(k . x - |k| t + phi) and its gradient
// (src/sevenpatch.jl:9-36) at the face nodes of the boundary faces.
struct WaveData {
    double k[3];
    double omega;
    double phi;
};

template <typename T>
struct FmArgs {
    const BlockItem* items;
    int nitems;
    int E;
    int mode;
    int truncate;
    T* u;
    T* y;
    T* acc;
    T* comp;
    T* du;
    const T* fu_in;     // u face exports of the current stage value (N^2 per slot)
    T* fu_out;
    T* V;               // (N^3, 3) per item: the fluxes F^d (V itself in the energy pass)
    T* fv;              // V face planes: (3, N^2) per slot
    const T* coef;      // (N^3, 10) per item
    const T* M;         // (N^3, 6) per item
    const T* rk;        // per problem dt/6, dt/3, dt/2, dt
    const double* tinfo;  // per problem: t_n, dt (FP64)
    const double* bnd_x;  // per slot: (3, N^2) physical positions of boundary face nodes
    WaveData wave;
    // truncation tables: per item slot (0 = the element's tensor projector)
    const int* eslot;
    const T* ew;        // ((P+1)^3, E^3, ntab)
    const T* echol;     // (P^3, P^3, E^3, ntab), upper factor U, G = U^T U
    double* partial;    // energy
    // the boundary faces' condition: 0 Dirichlet (the wave), 1 radiative
    int boundary;
    T kappa;
    T inv_r;
    // the factored truncation: per item 0 or 1 + its factored index f; per f
    // the radial dimension, the pair (P+1, E, nf), the angular table index;
    // the angular tables ((P+1)^2, E^2, ntab) and (P^2, P^2, E^2, ntab)
    const int* fslot;
    const int* fradial;
    const T* frm;
    const T* frd;
    const int* faslot;
    const T* faw;
    const T* fachol;
    // boundary kind 2: the caller's Dirichlet values (device table and the
    // boundary face index of every face slot)
    const int* bidx;
    const BoundaryTable* btab;
    // coarse-fine faces of a refined brick patch (flags bit f of an item):
    // u's ghosts (N^2 per slot) and V's ((3, N^2) per slot)
    const T* ugd;
    const T* vgd;
    // under a programmatic dependent launch: 1 where the pass lets the next
    // kernel launch from its start, 0 where it does so at its end
    int release;
};

template <typename T, int P>
struct FmTab {
    T L[P][P + 1];      // Legendre L_q at the Gauss-Lobatto nodes, q < P
};

__device__ __forceinline__ double stage_time(const double* tinfo, int problem, int mode) {
    const double c = mode == 1 || mode == 0 ? 0.0 : mode == 4 ? 1.0 : 0.5;
    return tinfo[2 * problem] + c * tinfo[2 * problem + 1];
}

// The caller's Dirichlet values of boundary face slot `slot` at time t: u,
// then the gradient's three Cartesian components, F values each. The level is
// the nearest to t; the host has checked that every stage time a call reaches
// is a level of the table, and the clamp only keeps the index in bounds.
template <typename T>
__device__ __forceinline__ const double* boundary_values(const FmArgs<T>& a, int slot, double t, int F) {
    const BoundaryTable bt = *a.btab;
    long long k = llrint((t - bt.t0) * bt.inv_half);
    k = k < 0 ? 0 : (k >= bt.nlevels ? bt.nlevels - 1 : k);
    return bt.values + ((k * bt.nbf + a.bidx[slot]) * 4) * (int64_t)F;
}

// The neighbour's tangential index of this face's point t = a + N b.
__device__ __forceinline__ int oriented(int t, int N, unsigned code) {
    int a = t % N, b = t / N;
    if (code & 1) { int s = a; a = b; b = s; }
    if (code & 2) a = N - 1 - a;
    if (code & 4) b = N - 1 - b;
    return a + N * b;
}

__device__ __forceinline__ unsigned face_orient(const BlockItem& it, int f) { return (it.orient >> (3 * f)) & 7u; }

__device__ __forceinline__ int sym_index(int d, int e) {
    // M^de in the order 00, 11, 22, 01, 02, 12
    return d == e ? d : d + e + 2;
}

// ---------------------------------------------------------------------------
// u's ghost across face f at its face node tt: a coarse-fine face's plane
// (the neighbour's u through I or R), the radiative face's own node (index
// `own` in the block, so that the wide derivative's face correction vanishes
// there, src/evolution.jl:1213-1221), the caller's Dirichlet value, the plane
// wave's value at the boundary face node's position, or the neighbour's
// exported face node, oriented across a glue.
template <typename T>
__device__ __forceinline__ T fm_u_ghost(const FmArgs<T>& a, const BlockItem& it, int f, int tt, int F, int N, double t,
                                        const T* yu, int own) {
    if (it.flags & (1u << f)) return a.ugd[(int64_t)(it.slot + f) * F + tt];
    if (it.nb[f] < 0 && a.boundary == 1) return yu[own];
    if (it.nb[f] < 0 && a.boundary == 2) return (T)boundary_values(a, it.slot + f, t, F)[tt];
    if (it.nb[f] < 0) {
        const double* X = a.bnd_x + (int64_t)(it.slot + f) * 3 * F;
        const double th = a.wave.k[0] * X[tt] + a.wave.k[1] * X[F + tt] + a.wave.k[2] * X[2 * F + tt] -
                          a.wave.omega * t + a.wave.phi;
        return (T)sin(th);
    }
    return a.fu_in[(int64_t)it.nb[f] * F + oriented(tt, N, face_orient(it, f))];
}

template <typename T, int P>
__global__ void __launch_bounds__(256) fm_gradient_kernel(FmArgs<T> a, Tab<T, P> tb) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    using G = ShapeR<3, P>;
    G g(a.E);
    constexpr int P1 = P + 1;
    T* su = reinterpret_cast<T*>(smem_raw);
    T* sD = su + g.SS;               // D_e u, ghost-free layout, e = 0, 1, 2
    const int mode = a.mode;
    const T* ysrc = (mode == MODE_RHS || mode == MODE_STAGE1 || mode == MODE_ENERGY) ? a.u : a.y;
    for (int item = blockIdx.x; item < a.nitems; item += gridDim.x) {
        const BlockItem& it = a.items[item];
        const T inv_h = T(1) / T(it.h);
        const double t = stage_time(a.tinfo, it.problem, mode == MODE_ENERGY ? 0 : mode);
        const T* yu = ysrc + it.off;
        if (threadIdx.x == 0) {
            // the flux coefficients and sqrt(g) stream into L2 while u loads
            prefetch_l2(a.M + (int64_t)item * 6 * g.NN, 6 * (size_t)g.NN * sizeof(T));
            prefetch_l2(a.coef + (int64_t)item * 10 * g.NN, (size_t)g.NN * sizeof(T));
        }
        for (int n = threadIdx.x; n < g.NN; n += blockDim.x) {
            int x[3];
            owned_coords<3>(g, n, x);
            su[sidx<3>(g, x)] = yu[n];
        }
        for (int i = threadIdx.x; i < 6 * g.F; i += blockDim.x) {
            const int f = i / g.F, tt = i % g.F;
            const int d = f >> 1, side = f & 1;
            int xo[3];
            plane_coords<3>(g, d, tt, side == 0 ? 0 : g.N - 1, xo);
            const T v = fm_u_ghost(a, it, f, tt, g.F, g.N, t, yu, oidx<3>(g, xo));
            int xg[3];
            plane_coords<3>(g, d, tt, side == 0 ? -1 : g.N, xg);
            su[sidx<3>(g, xg)] = v;
        }
        __syncthreads();
        // D_e u along every element line of every direction (one pass: the
        // three directions write three arrays)
        for (int L = threadIdx.x; L < 3 * g.E * g.F; L += blockDim.x) {
            const int e = L / (g.E * g.F), r = L % (g.E * g.F);
            const int tt = r % g.F, el = r / g.F;
            const int sd = g.sstride(e), ld = g.lstride(e);
            int x[3];
            plane_coords<3>(g, e, tt, el * P1, x);
            const int base = sidx<3>(g, x), lb = lidx<3>(g, x);
            T w[P + 3], out[P + 1];
#pragma unroll
            for (int k = 0; k < P + 3; ++k) w[k] = su[base + (k - 1) * sd];
            line_derivative<T, P>(tb, w, out);
            T* dst = sD + e * g.LS;
#pragma unroll
            for (int q = 0; q <= P; ++q) dst[lb + q * ld] = out[q];
        }
        __syncthreads();
        const T* cf = a.coef + (int64_t)item * 10 * g.NN;
        T* Vg = a.V + (int64_t)item * 3 * g.NN;
        if (mode == MODE_ENERGY) {
            // V = sum_e S[e] D_e u / (h sqrt(g)) at every node, for the energy
            for (int n = threadIdx.x; n < g.NN; n += blockDim.x) {
                int x[3];
                owned_coords<3>(g, n, x);
                const int l = lidx<3>(g, x);
                const T De[3] = {sD[l] * inv_h, sD[g.LS + l] * inv_h, sD[2 * g.LS + l] * inv_h};
                const T J = cf[n];
#pragma unroll
                for (int ci = 0; ci < 3; ++ci) {
                    T s = T(0);
#pragma unroll
                    for (int e = 0; e < 3; ++e) s += cf[(1 + 3 * e + ci) * g.NN + n] * De[e];
                    Vg[ci * g.NN + n] = s / J;
                }
            }
        } else {
            // the fluxes F^d = sum_e M^de D_e u / h at every node
            const T* Mb = a.M + (int64_t)item * 6 * g.NN;
            for (int n = threadIdx.x; n < g.NN; n += blockDim.x) {
                int x[3];
                owned_coords<3>(g, n, x);
                const int l = lidx<3>(g, x);
                const T De[3] = {sD[l] * inv_h, sD[g.LS + l] * inv_h, sD[2 * g.LS + l] * inv_h};
                T m[6];
#pragma unroll
                for (int k = 0; k < 6; ++k) m[k] = Mb[k * g.NN + n];
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    T s = T(0);
#pragma unroll
                    for (int e = 0; e < 3; ++e) s += m[sym_index(d, e)] * De[e];
                    Vg[d * g.NN + n] = s;
                }
            }
        }
        // V on the face planes for the neighbours
        for (int i = threadIdx.x; i < 6 * g.F; i += blockDim.x) {
            const int f = i / g.F, tt = i % g.F;
            const int d = f >> 1, side = f & 1;
            int x[3];
            plane_coords<3>(g, d, tt, side == 0 ? 0 : g.N - 1, x);
            const int l = lidx<3>(g, x), n = oidx<3>(g, x);
            const T De[3] = {sD[l] * inv_h, sD[g.LS + l] * inv_h, sD[2 * g.LS + l] * inv_h};
            const T J = cf[n];
            T* o = a.fv + (int64_t)(it.slot + f) * 3 * g.F;
#pragma unroll
            for (int ci = 0; ci < 3; ++ci) {
                T s = T(0);
#pragma unroll
                for (int e = 0; e < 3; ++e) s += cf[(1 + 3 * e + ci) * g.NN + n] * De[e];
                o[ci * g.F + tt] = s / J;
            }
        }
        __syncthreads();
    }
}

// The gradient pass with a compile-time block shape (E = 2 or 4): the
// register-line layout of stage3r_kernel. One thread per (a, b) position of
// the block's cross-section: its z column of u in registers, where it forms
// D_z u with the column's two ghosts; x and y lines from the padded shared
// copy of u, D_x into a ghost-free shared array and D_y kept in registers
// until every line has read u, then written over it. Each thread then forms
// the fluxes (or, in the energy pass, V) down its column, and the face planes
// of V read D_z on the x and y faces from a small plane buffer. Shared
// memory: u, D_x and the four planes, against u and three full arrays in the
// run-time-shape kernel.
template <typename T, int P, int E>
struct FmGradR {
    using S = Stage3R<T, P, E, false>;
    static constexpr size_t words = (size_t)S::SS + (size_t)S::LS + 4 * (size_t)S::F;
};

template <typename T, int P, int E>
__global__ void __launch_bounds__(Stage3R<T, P, E, false>::NT) fm_gradient_r_kernel(FmArgs<T> a, Tab<T, P> tb) {
    using S = Stage3R<T, P, E, false>;
    constexpr int N = S::N, F = S::F, NN = S::NN, VW = S::VW;
    constexpr int SX = S::SX, SXY = S::SXY, LX = S::LX, LXY = S::LXY;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* su = reinterpret_cast<T*>(smem_raw);   // padded u, then D_y (ghost-free layout)
    T* sx = su + S::SS;                      // D_x, ghost-free layout
    T* sz = sx + S::LS;                      // D_z on the nodes of faces 0-3, F each
    const int tid = threadIdx.x, ca = tid % N, cb = tid / N;
    const int s0 = 1 + SX * (ca + 1) + SXY * cb;   // x-line (x1, x2) = (ca, cb)
    const int s1 = (ca + 1) + SX + SXY * cb;       // y-line (x0, x2) = (ca, cb)
    const int s2 = (ca + 1) + SX * (cb + 1);       // z column (x0, x1) = (ca, cb)
    const int l0 = LX * ca + LXY * cb, l1 = ca + LXY * cb, l2 = ca + LX * cb;
    const int mode = a.mode;
    const T* ysrc = (mode == MODE_RHS || mode == MODE_STAGE1 || mode == MODE_ENERGY) ? a.u : a.y;
    // the block's metric (written once, at setup) into L2: the first block's
    // before the wait on the previous kernel
    auto prefetch = [&](int item) {
        prefetch_l2(a.M + (int64_t)item * 6 * NN, 6 * (size_t)NN * sizeof(T));
        prefetch_l2(a.coef + (int64_t)item * 10 * NN, (size_t)NN * sizeof(T));
    };
    if (tid == 0 && (int)blockIdx.x < a.nitems) prefetch(blockIdx.x);
    grid_dependency_wait();
    if (a.release) grid_dependents_launch();
    for (int item = blockIdx.x; item < a.nitems; item += gridDim.x) {
        const BlockItem& it = a.items[item];
        const T inv_h = T(1) / T(it.h);
        const double t = stage_time(a.tinfo, it.problem, mode == MODE_ENERGY ? 0 : mode);
        const T* yu = ysrc + it.off;
        if (tid == 0 && item != (int)blockIdx.x) prefetch(item);
        T line[N + 2];
#pragma unroll
        for (int j = 0; j < N; ++j) {
            line[1 + j] = yu[tid + F * j];
            su[s2 + SXY * j] = line[1 + j];
        }
        // this thread's ghosts: faces 0, 1 at its x line, 2, 3 at its y line
        // (tangential index tid on both), 4, 5 at its column
        su[s0 - 1] = fm_u_ghost(a, it, 0, tid, F, N, t, yu, N * ca + F * cb);
        su[s0 + N] = fm_u_ghost(a, it, 1, tid, F, N, t, yu, (N - 1) + N * ca + F * cb);
        su[s1 - SX] = fm_u_ghost(a, it, 2, tid, F, N, t, yu, ca + F * cb);
        su[s1 + N * SX] = fm_u_ghost(a, it, 3, tid, F, N, t, yu, ca + N * (N - 1) + F * cb);
        line[0] = fm_u_ghost(a, it, 4, tid, F, N, t, yu, tid);
        line[N + 1] = fm_u_ghost(a, it, 5, tid, F, N, t, yu, tid + F * (N - 1));
        T dz[N];
        line_full<T, P, E>(tb, line, dz, inv_h);
        // D_z on the x faces' nodes (0 or N-1, cb, j) and the y faces' (ca, 0 or N-1, j)
        if (ca == 0 || ca == N - 1) {
            T* o = sz + (ca == 0 ? 0 : F) + cb;
#pragma unroll
            for (int j = 0; j < N; ++j) o[N * j] = dz[j];
        }
        if (cb == 0 || cb == N - 1) {
            T* o = sz + (cb == 0 ? 2 * F : 3 * F) + ca;
#pragma unroll
            for (int j = 0; j < N; ++j) o[N * j] = dz[j];
        }
        __syncthreads();
        {
            // D_x along the x line, 16-byte loads of the contiguous padded row
            using V = typename V16<T>::type;
            T xl[N + 2], dx[N];
#pragma unroll
            for (int k = 0; k + VW <= N + 2; k += VW) {
                const V v = *reinterpret_cast<const V*>(su + s0 - 1 + k);
                const T* e = reinterpret_cast<const T*>(&v);
#pragma unroll
                for (int q = 0; q < VW; ++q) xl[k + q] = e[q];
            }
#pragma unroll
            for (int k = (N + 2) / VW * VW; k < N + 2; ++k) xl[k] = su[s0 - 1 + k];
            line_full<T, P, E>(tb, xl, dx, inv_h);
            if constexpr (N % VW == 0) {
#pragma unroll
                for (int j = 0; j < N; j += VW) {
                    V v;
                    T* e = reinterpret_cast<T*>(&v);
#pragma unroll
                    for (int q = 0; q < VW; ++q) e[q] = dx[j + q];
                    *reinterpret_cast<V*>(sx + l0 + j) = v;
                }
            } else {
#pragma unroll
                for (int j = 0; j < N; ++j) sx[l0 + j] = dx[j];
            }
        }
        T dy[N];
        {
            T yl[N + 2];
#pragma unroll
            for (int k = 0; k < N + 2; ++k) yl[k] = su[s1 + (k - 1) * SX];
            line_full<T, P, E>(tb, yl, dy, inv_h);
        }
        __syncthreads();   // every line has read u: D_y goes over it
#pragma unroll
        for (int j = 0; j < N; ++j) su[l1 + LX * j] = dy[j];
        __syncthreads();
        const T* cf = a.coef + (int64_t)item * 10 * NN;
        T* Vg = a.V + (int64_t)item * 3 * NN;
        if (mode == MODE_ENERGY) {
            // V = sum_e S[e] D_e u / (h sqrt(g)) at every node, for the energy
#pragma unroll 4
            for (int j = 0; j < N; ++j) {
                const int n = tid + F * j, l = l2 + LXY * j;
                const T De[3] = {sx[l], su[l], dz[j]};
                const T J = cf[n];
#pragma unroll
                for (int ci = 0; ci < 3; ++ci) {
                    T s = T(0);
#pragma unroll
                    for (int e = 0; e < 3; ++e) s += cf[(1 + 3 * e + ci) * NN + n] * De[e];
                    Vg[ci * NN + n] = s / J;
                }
            }
        } else {
            // the fluxes F^d = sum_e M^de D_e u / h at the column's nodes
            const T* Mb = a.M + (int64_t)item * 6 * NN;
#pragma unroll 4
            for (int j = 0; j < N; ++j) {
                const int n = tid + F * j, l = l2 + LXY * j;
                const T De[3] = {sx[l], su[l], dz[j]};
                T m[6];
#pragma unroll
                for (int k = 0; k < 6; ++k) m[k] = Mb[k * NN + n];
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    T s = T(0);
#pragma unroll
                    for (int e = 0; e < 3; ++e) s += m[sym_index(d, e)] * De[e];
                    Vg[d * NN + n] = s;
                }
            }
        }
        // V on the face planes for the neighbours: the x and y faces' nodes at
        // tangential index tid, and the column's own two z-face nodes
#pragma unroll
        for (int f = 0; f < 6; ++f) {
            const int side = f & 1;
            int x0, x1, x2;
            T dzf;
            if (f < 2) { x0 = side ? N - 1 : 0; x1 = ca; x2 = cb; dzf = sz[f * F + tid]; }
            else if (f < 4) { x0 = ca; x1 = side ? N - 1 : 0; x2 = cb; dzf = sz[f * F + tid]; }
            else { x0 = ca; x1 = cb; x2 = side ? N - 1 : 0; dzf = side ? dz[N - 1] : dz[0]; }
            const int l = x0 + LX * x1 + LXY * x2, n = x0 + N * x1 + F * x2;
            const T De[3] = {sx[l], su[l], dzf};
            const T J = cf[n];
            T* o = a.fv + (int64_t)(it.slot + f) * 3 * F;
#pragma unroll
            for (int ci = 0; ci < 3; ++ci) {
                T s = T(0);
#pragma unroll
                for (int e = 0; e < 3; ++e) s += cf[(1 + 3 * e + ci) * NN + n] * De[e];
                o[ci * F + tid] = s / J;
            }
        }
        __syncthreads();
    }
}

// sqrt(g)-orthogonal projection of v onto Q_{P-1} in one element (the ghost-free
// layout `sv`, element at x = base): c = Psi^T W v, U^T y = c, U z = y, v = Psi z
// (src/evolution.jl:384-425). cbuf holds P^3 coefficients per element.
template <typename T, int P, class G>
__device__ __forceinline__ void fm_project_block(const G& g, const FmArgs<T>& a, const T* L, int slot, T* sv,
                                                 T* cbuf) {
    constexpr int P1 = P + 1, n3 = P1 * P1 * P1, m3 = P * P * P;
    const int EE = g.E * g.E * g.E;
    const T* W = a.ew + (int64_t)slot * n3 * EE;
    const T* U = a.echol + (int64_t)slot * m3 * m3 * EE;
    // The element's node at (n0, n1, n2) in the ghost-free layout.
    auto at = [&](int e, int n0, int n1, int n2) {
        const int x[3] = {(e % g.E) * P1 + n0, ((e / g.E) % g.E) * P1 + n1, (e / (g.E * g.E)) * P1 + n2};
        return lidx<3>(g, x);
    };
    // c = Psi^T W v with Psi = L x L x L, one dimension at a time (sum
    // factorisation): each pass's thread owns one element line, reads its
    // P+1 values and writes its P results over the first P of them, so that
    // the passes work in place in the element's nodes; the last pass writes c.
    for (int i = threadIdx.x; i < EE * P1 * P1; i += blockDim.x) {     // along n0: (q0, n1, n2)
        const int e = i / (P1 * P1), n1 = i % P1, n2 = (i / P1) % P1;
        T t[P1];
#pragma unroll
        for (int n0 = 0; n0 < P1; ++n0)
            t[n0] = W[(int64_t)e * n3 + n0 + P1 * (n1 + P1 * n2)] * sv[at(e, n0, n1, n2)];
#pragma unroll
        for (int q0 = 0; q0 < P; ++q0) {
            T c = T(0);
#pragma unroll
            for (int n0 = 0; n0 < P1; ++n0) c += L[q0 * P1 + n0] * t[n0];
            sv[at(e, q0, n1, n2)] = c;
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < EE * P * P1; i += blockDim.x) {      // along n1: (q0, q1, n2)
        const int e = i / (P * P1), q0 = i % P, n2 = (i / P) % P1;
        T t[P1];
#pragma unroll
        for (int n1 = 0; n1 < P1; ++n1) t[n1] = sv[at(e, q0, n1, n2)];
#pragma unroll
        for (int q1 = 0; q1 < P; ++q1) {
            T c = T(0);
#pragma unroll
            for (int n1 = 0; n1 < P1; ++n1) c += L[q1 * P1 + n1] * t[n1];
            sv[at(e, q0, q1, n2)] = c;
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < EE * P * P; i += blockDim.x) {       // along n2: (q0, q1, q2)
        const int e = i / (P * P), q0 = i % P, q1 = (i / P) % P;
        T t[P1];
#pragma unroll
        for (int n2 = 0; n2 < P1; ++n2) t[n2] = sv[at(e, q0, q1, n2)];
#pragma unroll
        for (int q2 = 0; q2 < P; ++q2) {
            T c = T(0);
#pragma unroll
            for (int n2 = 0; n2 < P1; ++n2) c += L[q2 * P1 + n2] * t[n2];
            cbuf[e * m3 + q0 + P * (q1 + P * q2)] = c;
        }
    }
    __syncthreads();
    if (EE <= (int)blockDim.x) {
        // the triangular solves by every thread of the CTA: NG threads an
        // element, column by column, one barrier a column. At column q each
        // of an element's threads forms the unknown from its settled
        // right-hand side and subtracts its column from its own share of the
        // rows still open; the unknown is stored one column later, when no
        // thread reads that row any more.
        const int NG = blockDim.x / EE;
        const int e = threadIdx.x % EE, gl = threadIdx.x / EE;
        const bool act = gl < NG;
        T* c = cbuf + e * m3;
        const T* Ue = U + (int64_t)e * m3 * m3;   // column-major: U[r][q] at r + m3 q
        T prev = T(0);
        for (int q = 0; q < m3; ++q) {            // U^T y = c
            if (act) {
                const T y = c[q] / Ue[q + m3 * q];
                if (q > 0 && gl == (q - 1) % NG) c[q - 1] = prev;
                for (int r = q + 1 + gl; r < m3; r += NG) c[r] -= Ue[q + m3 * r] * y;
                prev = y;
            }
            __syncthreads();
        }
        if (act && gl == (m3 - 1) % NG) c[m3 - 1] = prev;
        __syncthreads();
        for (int q = m3 - 1; q >= 0; --q) {       // U z = y
            if (act) {
                const T z = c[q] / Ue[q + m3 * q];
                if (q < m3 - 1 && gl == (q + 1) % NG) c[q + 1] = prev;
                for (int r = gl; r < q; r += NG) c[r] -= Ue[r + m3 * q] * z;
                prev = z;
            }
            __syncthreads();
        }
        if (act && gl == 0) c[0] = prev;
    } else {
        for (int e = threadIdx.x; e < EE; e += blockDim.x) {
            T* c = cbuf + e * m3;
            const T* Ue = U + (int64_t)e * m3 * m3;   // column-major: U[r][q] at r + m3 q
            for (int q = 0; q < m3; ++q) {            // U^T y = c
                T s = c[q];
                for (int r = 0; r < q; ++r) s -= Ue[r + m3 * q] * c[r];
                c[q] = s / Ue[q + m3 * q];
            }
            for (int q = m3 - 1; q >= 0; --q) {       // U z = y
                T s = c[q];
                for (int r = q + 1; r < m3; ++r) s -= Ue[q + m3 * r] * c[r];
                c[q] = s / Ue[q + m3 * q];
            }
        }
    }
    __syncthreads();
    // v = Psi z, the same passes backwards: from c along q2 into the
    // element's nodes (q0, q1, n2), then along q1 and q0, each line's thread
    // reading its P values before it writes its P+1
    for (int i = threadIdx.x; i < EE * P * P; i += blockDim.x) {       // along q2: (q0, q1, n2)
        const int e = i / (P * P), q0 = i % P, q1 = (i / P) % P;
        T t[P];
#pragma unroll
        for (int q2 = 0; q2 < P; ++q2) t[q2] = cbuf[e * m3 + q0 + P * (q1 + P * q2)];
#pragma unroll
        for (int n2 = 0; n2 < P1; ++n2) {
            T z = T(0);
#pragma unroll
            for (int q2 = 0; q2 < P; ++q2) z += L[q2 * P1 + n2] * t[q2];
            sv[at(e, q0, q1, n2)] = z;
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < EE * P * P1; i += blockDim.x) {      // along q1: (q0, n1, n2)
        const int e = i / (P * P1), q0 = i % P, n2 = (i / P) % P1;
        T t[P];
#pragma unroll
        for (int q1 = 0; q1 < P; ++q1) t[q1] = sv[at(e, q0, q1, n2)];
#pragma unroll
        for (int n1 = 0; n1 < P1; ++n1) {
            T z = T(0);
#pragma unroll
            for (int q1 = 0; q1 < P; ++q1) z += L[q1 * P1 + n1] * t[q1];
            sv[at(e, q0, n1, n2)] = z;
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < EE * P1 * P1; i += blockDim.x) {     // along q0: (n0, n1, n2)
        const int e = i / (P1 * P1), n1 = i % P1, n2 = (i / P1) % P1;
        T t[P];
#pragma unroll
        for (int q0 = 0; q0 < P; ++q0) t[q0] = sv[at(e, q0, n1, n2)];
#pragma unroll
        for (int n0 = 0; n0 < P1; ++n0) {
            T z = T(0);
#pragma unroll
            for (int q0 = 0; q0 < P; ++q0) z += L[q0 * P1 + n0] * t[q0];
            sv[at(e, n0, n1, n2)] = z;
        }
    }
    __syncthreads();
}

// The factored truncation of one block (src/evolution.jl:308-382): along the
// radial dimension k the rank-one pair of each element line, then on each of
// an element's P+1 planes across k the 2D sqrt(g)-orthogonal projection with
// the angular tables: c = Psi^T W v, U^T y = c, U z = y, v = Psi z. The two
// act on different indices and their product is the projection onto Q_{P-1}.
// The node of an element with index jk along dimension k and (ja, jb) along
// the two others in increasing order, as an index into the ghost-free
// layout; selects only, so that nothing indexes a local array at run time.
template <class G>
__device__ __forceinline__ int node_across(const G& g, int k, int jk, int ja, int jb) {
    int x[3];
    x[0] = k == 0 ? jk : ja;
    x[1] = k == 1 ? jk : (k == 0 ? ja : jb);
    x[2] = k == 2 ? jk : jb;
    return lidx<3>(g, x);
}

__device__ __forceinline__ int pick3(int k, int a0, int a1, int a2) { return k == 0 ? a0 : k == 1 ? a1 : a2; }

template <typename T, int P, class G>
__device__ __forceinline__ void fm_project_factored(const G& g, const FmArgs<T>& a, const T* L, int f, T* sv,
                                                    T* cbuf) {
    constexpr int P1 = P + 1, n2 = P1 * P1, m2 = P * P;
    const int E = g.E, EE = E * E * E, E2 = E * E;
    const int k = a.fradial[f], A = a.faslot[f];
    const int d0 = k == 0 ? 1 : 0, d1 = k == 2 ? 1 : 2;
    const int ls = g.lstride(k);
    // along k: v -= mode (dual . v) on every element line
    for (int i = threadIdx.x; i < EE * n2; i += blockDim.x) {
        const int e = i / n2, nn = i % n2;
        const int e0 = e % E, e1 = (e / E) % E, e2 = e / E2;
        const int ek = pick3(k, e0, e1, e2), ea = pick3(d0, e0, e1, e2), eb = pick3(d1, e0, e1, e2);
        const T* rm = a.frm + ((int64_t)f * E + ek) * P1;
        const T* rd = a.frd + ((int64_t)f * E + ek) * P1;
        const int l0 = node_across(g, k, ek * P1, ea * P1 + nn % P1, eb * P1 + nn / P1);
        T v[P1];
        T c = T(0);
#pragma unroll
        for (int j = 0; j < P1; ++j) { v[j] = sv[l0 + j * ls]; c += rd[j] * v[j]; }
#pragma unroll
        for (int j = 0; j < P1; ++j) sv[l0 + j * ls] = v[j] - rm[j] * c;
    }
    __syncthreads();
    // across k, plane by plane, one thread a plane of an element: c = Psi^T W v
    // with Psi = L x L summed one dimension at a time, the Cholesky solves
    // U^T y = c, U z = y, and v = Psi z back the same way, all in registers;
    // the planes are disjoint, so no barrier separates the steps
    for (int u = threadIdx.x; u < EE * P1; u += blockDim.x) {
        const int e = u / P1, j = u % P1;
        const int e0 = e % E, e1 = (e / E) % E, e2 = e / E2;
        const int ek = pick3(k, e0, e1, e2), ea = pick3(d0, e0, e1, e2), eb = pick3(d1, e0, e1, e2);
        const T* W = a.faw + ((int64_t)A * E2 + ea + E * eb) * n2;
        const T* U = a.fachol + ((int64_t)A * E2 + ea + E * eb) * m2 * m2;   // U[r][q] at r + m2 q
        T t[P1][P1];
#pragma unroll
        for (int nb = 0; nb < P1; ++nb)
#pragma unroll
            for (int na = 0; na < P1; ++na)
                t[nb][na] = W[na + P1 * nb] * sv[node_across(g, k, ek * P1 + j, ea * P1 + na, eb * P1 + nb)];
        T c[m2];
        {
            T A0[P1][P];   // A0[nb][q0] = sum_na L_q0(na) t[nb][na]
#pragma unroll
            for (int nb = 0; nb < P1; ++nb)
#pragma unroll
                for (int q0 = 0; q0 < P; ++q0) {
                    T s = T(0);
#pragma unroll
                    for (int na = 0; na < P1; ++na) s += L[q0 * P1 + na] * t[nb][na];
                    A0[nb][q0] = s;
                }
#pragma unroll
            for (int q1 = 0; q1 < P; ++q1)
#pragma unroll
                for (int q0 = 0; q0 < P; ++q0) {
                    T s = T(0);
#pragma unroll
                    for (int nb = 0; nb < P1; ++nb) s += L[q1 * P1 + nb] * A0[nb][q0];
                    c[q0 + P * q1] = s;
                }
        }
#pragma unroll
        for (int q = 0; q < m2; ++q) {            // U^T y = c
            T s = c[q];
#pragma unroll
            for (int r = 0; r < q; ++r) s -= U[r + m2 * q] * c[r];
            c[q] = s / U[q + m2 * q];
        }
#pragma unroll
        for (int q = m2 - 1; q >= 0; --q) {       // U z = y
            T s = c[q];
#pragma unroll
            for (int r = q + 1; r < m2; ++r) s -= U[q + m2 * r] * c[r];
            c[q] = s / U[q + m2 * q];
        }
        {
            T B0[P1][P];   // B0[nb][q0] = sum_q1 L_q1(nb) z[q0 + P q1]
#pragma unroll
            for (int nb = 0; nb < P1; ++nb)
#pragma unroll
                for (int q0 = 0; q0 < P; ++q0) {
                    T s = T(0);
#pragma unroll
                    for (int q1 = 0; q1 < P; ++q1) s += L[q1 * P1 + nb] * c[q0 + P * q1];
                    B0[nb][q0] = s;
                }
#pragma unroll
            for (int nb = 0; nb < P1; ++nb)
#pragma unroll
                for (int na = 0; na < P1; ++na) {
                    T z = T(0);
#pragma unroll
                    for (int q0 = 0; q0 < P; ++q0) z += L[q0 * P1 + na] * B0[nb][q0];
                    sv[node_across(g, k, ek * P1 + j, ea * P1 + na, eb * P1 + nb)] = z;
                }
        }
    }
    __syncthreads();
}

// The truncation of one block of the full metric: the element's tensor
// projector (affine patch), the per-element projection, or the factored one.
template <typename T, int P, class G>
__device__ __forceinline__ void fm_truncate_block(const G& g, const FmArgs<T>& a, const Tab<T, P>& tb, const T* L,
                                                  int item, T* sv, T* cbuf) {
    const int s = a.eslot[item];
    const int f = a.fslot ? a.fslot[item] : 0;
    if (s > 0) fm_project_block<T, P>(g, a, L, s - 1, sv, cbuf);
    else if (f > 0) fm_project_factored<T, P>(g, a, L, f - 1, sv, cbuf);
    else truncate_block<T, 3, P, false, 0>(g, tb, sv, nullptr);
}

// The Legendre table in shared memory (a kernel-parameter array indexed at
// run time would be copied to local memory): L[q (P+1) + i] = L_q(node i).
template <typename T, int P>
__device__ __forceinline__ void stage_legendre(const FmTab<T, P>& ft, T* L) {
    for (int i = threadIdx.x; i < P * (P + 1); i += blockDim.x) {
        const int q = i / (P + 1), n = i % (P + 1);
#pragma unroll
        for (int qq = 0; qq < P; ++qq)
#pragma unroll
            for (int nn = 0; nn <= P; ++nn)
                if (qq == q && nn == n) L[i] = ft.L[qq][nn];
    }
    __syncthreads();
}

// FM: the stage the instantiation runs (1-4), so that each stage's code holds
// only its own data flow, or 0 for the mode in the arguments.
// The flux F^d = S[d] . V beyond face f (normal d, side) at its face node tt,
// with this face node's own S[d] (node `o` of the block): the neighbour's
// exported V, oriented across a glue; a coarse-fine face's plane; the
// caller's Dirichlet gradient; the plane wave's gradient at the boundary face
// node; or on the radiative sphere 2 F* - F, so that the central flux through
// the face is F* = -sigma |S[d]| (kappa v + u / R) (src/evolution.jl:1232-1260).
template <typename T>
__device__ __forceinline__ T fm_flux_ghost(const FmArgs<T>& a, const BlockItem& it, int f, int d, int side, int tt,
                                           int o, int F, int N, int NN, double t, const T* cf, const T* Fb,
                                           const T* ysrc) {
    if (it.nb[f] < 0 && !(it.flags & (1u << f)) && a.boundary == 1) {
        const T Fo = Fb[d * NN + o];
        T S2 = T(0);
#pragma unroll
        for (int ci = 0; ci < 3; ++ci) {
            const T Sc = cf[(1 + 3 * d + ci) * NN + o];
            S2 += Sc * Sc;
        }
        const T* yo = ysrc + it.off;
        const T sigma = side ? T(1) : T(-1);
        const T Fstar = -sigma * sqrt(S2) * (a.kappa * yo[NN + o] + a.inv_r * yo[o]);
        return T(2) * Fstar - Fo;
    }
    T Vg[3];
    if (it.flags & (1u << f)) {
        const T* src = a.vgd + (int64_t)(it.slot + f) * 3 * F;
#pragma unroll
        for (int ci = 0; ci < 3; ++ci) Vg[ci] = src[ci * F + tt];
    } else if (it.nb[f] < 0 && a.boundary == 2) {
        const double* bv = boundary_values(a, it.slot + f, t, F);
#pragma unroll
        for (int ci = 0; ci < 3; ++ci) Vg[ci] = (T)bv[(1 + ci) * F + tt];
    } else if (it.nb[f] < 0) {
        const double* X = a.bnd_x + (int64_t)(it.slot + f) * 3 * F;
        const double th = a.wave.k[0] * X[tt] + a.wave.k[1] * X[F + tt] + a.wave.k[2] * X[2 * F + tt] -
                          a.wave.omega * t + a.wave.phi;
        const double c = cos(th);
#pragma unroll
        for (int ci = 0; ci < 3; ++ci) Vg[ci] = (T)(a.wave.k[ci] * c);
    } else {
        const T* src = a.fv + (int64_t)it.nb[f] * 3 * F;
        const int t2 = oriented(tt, N, face_orient(it, f));
#pragma unroll
        for (int ci = 0; ci < 3; ++ci) Vg[ci] = src[ci * F + t2];
    }
    T Fg = T(0);
#pragma unroll
    for (int ci = 0; ci < 3; ++ci) Fg += cf[(1 + 3 * d + ci) * NN + o] * Vg[ci];
    return Fg;
}

template <typename T, int P, bool COMP, int FM = 0>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 3 : 4) fm_stage_kernel(FmArgs<T> a, Tab<T, P> tb, FmTab<T, P> ft) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    using G = ShapeR<3, P>;
    G g(a.E);
    constexpr int P1 = P + 1;
    T* sF = reinterpret_cast<T*>(smem_raw);   // flux along the current d, padded
    T* sl = sF + g.SS;                        // Laplacian accumulator, then the new v
    T* sc = sl + g.LS;                        // compensation of v (COMP)
    T* cbuf = sc + g.LS;                      // truncation coefficients
    __shared__ T sLeg[P * (P + 1)];
    stage_legendre<T, P>(ft, sLeg);
    const int mode = FM ? FM : a.mode;
    const T* ysrc = (mode == MODE_RHS || mode == MODE_STAGE1) ? a.u : a.y;
    for (int item = blockIdx.x; item < a.nitems; item += gridDim.x) {
        const BlockItem& it = a.items[item];
        const T inv_h = T(1) / T(it.h);
        const double t = stage_time(a.tinfo, it.problem, mode);
        const T* cf = a.coef + (int64_t)item * 10 * g.NN;
        const T* Fb = a.V + (int64_t)item * 3 * g.NN;
        if (threadIdx.x == 0) {
            // everything the block reads after its fluxes: sqrt(g), the RK
            // operands and its truncation tables, into L2 while the fluxes load
            const size_t b = (size_t)g.NN * sizeof(T);
            prefetch_l2(Fb, 3 * b);
            prefetch_l2(cf, b);
            prefetch_l2(ysrc + it.off, 2 * b);
            if (mode != MODE_RHS && mode != MODE_STAGE1) {
                prefetch_l2(a.u + it.off, 2 * b);
                prefetch_l2(a.acc + it.off, 2 * b);
                if (COMP && mode == MODE_STAGE4) prefetch_l2(a.comp + it.off, 2 * b);
            }
            const int es = a.eslot[item];
            if (a.truncate && es > 0) {
                constexpr int n3 = (P + 1) * (P + 1) * (P + 1), m3 = P * P * P;
                const size_t EE = (size_t)g.E * g.E * g.E;
                prefetch_l2(a.ew + (int64_t)(es - 1) * n3 * EE, n3 * EE * sizeof(T));
                prefetch_l2(a.echol + (int64_t)(es - 1) * m3 * m3 * EE, (size_t)m3 * m3 * EE * sizeof(T));
            }
        }
        for (int d = 0; d < 3; ++d) {
            const int sd = g.sstride(d), ld = g.lstride(d);
            // F^d at the owned nodes, from the gradient pass
            for (int n = threadIdx.x; n < g.NN; n += blockDim.x) {
                int x[3];
                owned_coords<3>(g, n, x);
                sF[sidx<3>(g, x)] = Fb[d * g.NN + n];
            }
            // ... and at the two ghost planes along d, with the face node's S[d]
            for (int i = threadIdx.x; i < 2 * g.F; i += blockDim.x) {
                const int side = i / g.F, tt = i % g.F;
                const int f = 2 * d + side;
                int xo[3], xg[3];
                plane_coords<3>(g, d, tt, side == 0 ? 0 : g.N - 1, xo);
                plane_coords<3>(g, d, tt, side == 0 ? -1 : g.N, xg);
                const int o = oidx<3>(g, xo);
                sF[sidx<3>(g, xg)] = fm_flux_ghost(a, it, f, d, side, tt, o, g.F, g.N, g.NN, t, cf, Fb, ysrc);
            }
            __syncthreads();
            for (int L = threadIdx.x; L < g.E * g.F; L += blockDim.x) {
                const int tt = L % g.F, el = L / g.F;
                int x[3];
                plane_coords<3>(g, d, tt, el * P1, x);
                const int base = sidx<3>(g, x), lb = lidx<3>(g, x);
                T w[P + 3], out[P + 1];
#pragma unroll
                for (int k = 0; k < P + 3; ++k) w[k] = sF[base + (k - 1) * sd];
                line_derivative<T, P>(tb, w, out);
#pragma unroll
                for (int q = 0; q <= P; ++q) {
                    if (d == 0) sl[lb + q * ld] = out[q];
                    else sl[lb + q * ld] += out[q];
                }
            }
            __syncthreads();
        }
        const T* yv = ysrc + it.off + g.NN;
        if (mode == MODE_RHS) {
            T* du = a.du + it.off;
            for (int n = threadIdx.x; n < g.NN; n += blockDim.x) {
                int x[3];
                owned_coords<3>(g, n, x);
                du[n] = yv[n];
                du[g.NN + n] = sl[lidx<3>(g, x)] * inv_h / cf[n];
            }
            __syncthreads();
            continue;
        }
        const RkCoef<T> rc(mode, a.rk + 4 * it.problem);
        const T* un = a.u + it.off;
        T* acc = a.acc + it.off;
        T* comp = COMP ? a.comp + it.off : nullptr;
        const bool final_comp = COMP && mode == MODE_STAGE4;
        T* out = (mode == MODE_STAGE4 ? a.u : a.y) + it.off;
        for (int n = threadIdx.x; n < g.NN; n += blockDim.x) {
            int x[3];
            owned_coords<3>(g, n, x);
            const int l = lidx<3>(g, x);
            T lap[1] = {sl[l] / cf[n]};
            T yq[1] = {yv[n]}, uuq[1] = {un[n]}, uvq[1] = {un[g.NN + n]}, auq[1], avq[1], cuq[1], cviq[1];
            if (mode != 1) { auq[0] = acc[n]; avq[0] = acc[g.NN + n]; }
            if (final_comp) { cuq[0] = comp[n]; cviq[0] = comp[g.NN + n]; }
            T nu[1], nv[1], cv[1];
            stage_points<T, COMP, 1>(mode, rc, yq, uuq, uvq, auq, avq, cuq, cviq, lap, inv_h, nu, nv, cv);
            if (mode != MODE_STAGE4) { acc[n] = auq[0]; acc[g.NN + n] = avq[0]; }
            if (final_comp) { comp[n] = cuq[0]; sc[l] = cv[0]; }
            out[n] = nu[0];
            sl[l] = nv[0];
        }
        __syncthreads();
        if (a.truncate) {
            fm_truncate_block<T, P>(g, a, tb, sLeg, item, sl, cbuf);
            if (final_comp) fm_truncate_block<T, P>(g, a, tb, sLeg, item, sc, cbuf);
        }
        for (int n = threadIdx.x; n < g.NN; n += blockDim.x) {
            int x[3];
            owned_coords<3>(g, n, x);
            out[g.NN + n] = sl[lidx<3>(g, x)];
            if (final_comp) comp[g.NN + n] = sc[lidx<3>(g, x)];
        }
        // u's face nodes of the new stage value for the next gradient pass
        for (int i = threadIdx.x; i < 6 * g.F; i += blockDim.x) {
            const int f = i / g.F, tt = i % g.F;
            const int d = f >> 1, side = f & 1;
            int x[3];
            plane_coords<3>(g, d, tt, side == 0 ? 0 : g.N - 1, x);
            a.fu_out[(int64_t)(it.slot + f) * g.F + tt] = out[oidx<3>(g, x)];
        }
        __syncthreads();
    }
}

// The stage pass with a compile-time block shape (E = 2 or 4) in the
// register-line layout (fmstage_r.cuh), instantiated per order in a
// translation unit of its own (kernels_d3_p<P>_fm.cu): its shared-memory
// attributes, its shared memory in bytes, and a launch of RK stage `mode`.
template <typename T, int P, int E, bool COMP>
void fm_stage_r_attrs(int max_smem);
template <typename T, int P, int E, bool COMP>
size_t fm_stage_r_smem();
template <typename T, int P, int E, bool COMP>
cudaError_t fm_stage_r_launch(const FmArgs<T>& a, const Tab<T, P>& tb, const FmTab<T, P>& ft, int grid, int mode,
                              cudaStream_t s, bool pdl);

// The standalone truncation of the full metric (twoldg_truncate).
template <typename T, int P>
__global__ void __launch_bounds__(256) fm_truncate_kernel(FmArgs<T> a, Tab<T, P> tb, FmTab<T, P> ft) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    using G = ShapeR<3, P>;
    G g(a.E);
    T* sv = reinterpret_cast<T*>(smem_raw);
    T* cbuf = sv + g.LS;
    __shared__ T sLeg[P * (P + 1)];
    stage_legendre<T, P>(ft, sLeg);
    for (int item = blockIdx.x; item < a.nitems; item += gridDim.x) {
        T* v = a.u + a.items[item].off + g.NN;
        for (int n = threadIdx.x; n < g.NN; n += blockDim.x) {
            int x[3];
            owned_coords<3>(g, n, x);
            sv[lidx<3>(g, x)] = v[n];
        }
        __syncthreads();
        fm_truncate_block<T, P>(g, a, tb, sLeg, item, sv, cbuf);
        for (int n = threadIdx.x; n < g.NN; n += blockDim.x) {
            int x[3];
            owned_coords<3>(g, n, x);
            v[n] = sv[lidx<3>(g, x)];
        }
        __syncthreads();
    }
}

// The full metric's energy, 1/2 sum w sqrt(g) (v^2 + |V|^2) (src/evolution.jl:1472-1489),
// from V of the last gradient pass; one FP64 partial per block.
template <typename T, int P>
__global__ void __launch_bounds__(256) fm_energy_kernel(FmArgs<T> a, Tab<T, P> tb) {
    __shared__ double red[32];
    using G = ShapeR<3, P>;
    G g(a.E);
    constexpr int P1 = P + 1;
    for (int item = blockIdx.x; item < a.nitems; item += gridDim.x) {
        const BlockItem& it = a.items[item];
        const double wscale = it.h * P1 / 2.0;
        const T* cf = a.coef + (int64_t)item * 10 * g.NN;
        const T* Vb = a.V + (int64_t)item * 3 * g.NN;
        const T* v = a.u + it.off + g.NN;
        double local = 0;
        for (int n = threadIdx.x; n < g.NN; n += blockDim.x) {
            int x[3];
            owned_coords<3>(g, n, x);
            double w = 1.0;
            for (int k = 0; k < 3; ++k) w *= wscale * (double)tb.wq[x[k] % P1];
            double s = (double)v[n] * (double)v[n];
            for (int ci = 0; ci < 3; ++ci) s += (double)Vb[ci * g.NN + n] * (double)Vb[ci * g.NN + n];
            local += w * (double)cf[n] * s;
        }
        // a radiative boundary's own energy, 1/2 inv_r sum w |S[d]| u^2 over its
        // faces' nodes (src/evolution.jl:1265-1288)
        if (a.boundary == 1 && a.inv_r != T(0)) {
            const T* uu = a.u + it.off;
            for (int i = threadIdx.x; i < 6 * g.F; i += blockDim.x) {
                const int f = i / g.F, tt = i % g.F;
                if (it.nb[f] >= 0 || (it.flags & (1u << f))) continue;
                const int d = f >> 1, side = f & 1;
                int x[3];
                plane_coords<3>(g, d, tt, side == 0 ? 0 : g.N - 1, x);
                const int o = oidx<3>(g, x);
                double w = 1.0;
                for (int q = 0; q < 3; ++q)
                    if (q != d) w *= wscale * (double)tb.wq[x[q] % P1];
                double S2 = 0;
                for (int ci = 0; ci < 3; ++ci) {
                    const double Sc = (double)cf[(1 + 3 * d + ci) * g.NN + o];
                    S2 += Sc * Sc;
                }
                local += w * sqrt(S2) * (double)uu[o] * (double)uu[o] * (double)a.inv_r;
            }
        }
        double s = block_reduce_sum<3>(local, red);
        if (threadIdx.x == 0) a.partial[item] = 0.5 * s;
        __syncthreads();
    }
}

}  // namespace twoldg
