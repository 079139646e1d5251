// The full-metric field step (3D): a geometry whose glues may swap axes,
// such as the seven-patch ball (src/evolution.jl:112-220, 266-425,
// 1110-1127). The gradient crosses faces as Cartesian components
// V = grad u, all three in one field with a ghost plane on every face, so
// a stage is two passes:
//   fm_gradient_kernel: V_i = sum_e S[e][i] D_e u / (h sqrt(g)) at every node
//     (u's face ghosts from the neighbours' exported face nodes, oriented
//     across the glue, or the Dirichlet data on the domain's boundary), and
//     V's face planes for the neighbours;
//   fm_stage_kernel: sqrt(g) v' = sum_d D_d F^d with the flux F^d = S[d] . V
//     formed at every point of the window along d, the ghost's with the face
//     node's own S[d]; then the RK combination, the sqrt(g)-orthogonal
//     truncation of v per element (Cholesky solves, or the element's tensor
//     projector on an affine patch) and u's face export.
// coef holds, per block, (N^3, 10): sqrt(g), then S[d][i] at 1 + 3d + i.
#pragma once

#include "kernels.cuh"

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
    T* V;               // (N^3, 3) per item
    T* fv;              // V face planes: (3, N^2) per slot
    const T* coef;      // (N^3, 10) per item
    const T* rk;        // per problem dt/6, dt/3, dt/2, dt
    const double* tinfo;  // per problem: t_n, dt (FP64)
    const double* bnd_x;  // per slot: (3, N^2) physical positions of boundary face nodes
    WaveData wave;
    // truncation tables: per item slot (0 = the element's tensor projector)
    const int* eslot;
    const T* ew;        // ((P+1)^3, E^3, ntab)
    const T* echol;     // (P^3, P^3, E^3, ntab), upper factor U, G = U^T U
    double* partial;    // energy
};

template <typename T, int P>
struct FmTab {
    T L[P][P + 1];      // Legendre L_q at the Gauss-Lobatto nodes, q < P
};

__device__ __forceinline__ double stage_time(const double* tinfo, int problem, int mode) {
    const double c = mode == 1 || mode == 0 ? 0.0 : mode == 4 ? 1.0 : 0.5;
    return tinfo[2 * problem] + c * tinfo[2 * problem + 1];
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

// ---------------------------------------------------------------------------
template <typename T, int P>
__global__ void __launch_bounds__(256) fm_gradient_kernel(FmArgs<T> a, Tab<T, P> tb) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    using G = ShapeR<3, P>;
    G g(a.E);
    constexpr int P1 = P + 1;
    T* su = reinterpret_cast<T*>(smem_raw);
    T* sv = su + g.SS;               // V, ghost-free layout, 3 components
    const int mode = a.mode;
    const T* ysrc = (mode == MODE_RHS || mode == MODE_STAGE1 || mode == MODE_ENERGY) ? a.u : a.y;
    for (int item = blockIdx.x; item < a.nitems; item += gridDim.x) {
        const BlockItem& it = a.items[item];
        const T inv_h = T(1) / T(it.h);
        const double t = stage_time(a.tinfo, it.problem, mode == MODE_ENERGY ? 0 : mode);
        const T* yu = ysrc + it.off;
        for (int n = threadIdx.x; n < g.NN; n += blockDim.x) {
            int x[3];
            owned_coords<3>(g, n, x);
            su[sidx<3>(g, x)] = yu[n];
        }
        for (int i = threadIdx.x; i < 6 * g.F; i += blockDim.x) {
            const int f = i / g.F, tt = i % g.F;
            const int d = f >> 1, side = f & 1;
            T v;
            if (it.nb[f] < 0) {
                // Dirichlet: the data at the boundary face node's position
                const double* X = a.bnd_x + (int64_t)(it.slot + f) * 3 * g.F;
                const double th = a.wave.k[0] * X[tt] + a.wave.k[1] * X[g.F + tt] + a.wave.k[2] * X[2 * g.F + tt] -
                                  a.wave.omega * t + a.wave.phi;
                v = (T)sin(th);
            } else {
                v = a.fu_in[(int64_t)it.nb[f] * g.F + oriented(tt, g.N, face_orient(it, f))];
            }
            int xg[3];
            plane_coords<3>(g, d, tt, side == 0 ? -1 : g.N, xg);
            su[sidx<3>(g, xg)] = v;
        }
        __syncthreads();
        const T* cf = a.coef + (int64_t)item * 10 * g.NN;
        for (int n = threadIdx.x; n < 3 * g.LS; n += blockDim.x) sv[n] = T(0);
        __syncthreads();
        // V_i += S[e][i] D_e u / h, line by line along e
        for (int e = 0; e < 3; ++e) {
            const int sd = g.sstride(e);
            const int od = e == 0 ? 1 : e == 1 ? g.N : g.N * g.N;
            const int ld = g.lstride(e);
            for (int L = threadIdx.x; L < g.E * g.F; L += blockDim.x) {
                const int tt = L % g.F, el = L / g.F;
                int x[3];
                plane_coords<3>(g, e, tt, el * P1, x);
                const int base = sidx<3>(g, x), ob = oidx<3>(g, x), lb = lidx<3>(g, x);
                T w[P + 3], out[P + 1];
#pragma unroll
                for (int k = 0; k < P + 3; ++k) w[k] = su[base + (k - 1) * sd];
                line_derivative<T, P>(tb, w, out);
#pragma unroll
                for (int q = 0; q <= P; ++q) {
                    const T De = out[q] * inv_h;
                    const int o = ob + q * od;
#pragma unroll
                    for (int ci = 0; ci < 3; ++ci) sv[ci * g.LS + lb + q * ld] += cf[(1 + 3 * e + ci) * g.NN + o] * De;
                }
            }
            __syncthreads();
        }
        T* Vg = a.V + (int64_t)item * 3 * g.NN;
        for (int n = threadIdx.x; n < g.NN; n += blockDim.x) {
            int x[3];
            owned_coords<3>(g, n, x);
            const int l = lidx<3>(g, x);
            const T J = cf[n];
#pragma unroll
            for (int ci = 0; ci < 3; ++ci) {
                const T val = sv[ci * g.LS + l] / J;
                sv[ci * g.LS + l] = val;
                Vg[ci * g.NN + n] = val;
            }
        }
        __syncthreads();
        // V's face planes for the neighbours
        for (int i = threadIdx.x; i < 6 * g.F; i += blockDim.x) {
            const int f = i / g.F, tt = i % g.F;
            const int d = f >> 1, side = f & 1;
            int x[3];
            plane_coords<3>(g, d, tt, side == 0 ? 0 : g.N - 1, x);
            const int l = lidx<3>(g, x);
            T* o = a.fv + (int64_t)(it.slot + f) * 3 * g.F;
#pragma unroll
            for (int ci = 0; ci < 3; ++ci) o[ci * g.F + tt] = sv[ci * g.LS + l];
        }
        __syncthreads();
    }
}

// sqrt(g)-orthogonal projection of v onto Q_{P-1} in one element (the ghost-free
// layout `sv`, element at x = base): c = Psi^T W v, U^T y = c, U z = y, v = Psi z
// (src/evolution.jl:384-425). cbuf holds P^3 coefficients per element.
template <typename T, int P, class G>
__device__ __forceinline__ void fm_project_block(const G& g, const FmArgs<T>& a, const FmTab<T, P>& ft, int slot,
                                                 T* sv, T* cbuf) {
    constexpr int P1 = P + 1, n3 = P1 * P1 * P1, m3 = P * P * P;
    const int EE = g.E * g.E * g.E;
    const T* W = a.ew + (int64_t)slot * n3 * EE;
    const T* U = a.echol + (int64_t)slot * m3 * m3 * EE;
    for (int i = threadIdx.x; i < EE * m3; i += blockDim.x) {
        const int e = i / m3, q = i % m3;
        const int q0 = q % P, q1 = (q / P) % P, q2 = q / (P * P);
        const int e0 = e % g.E, e1 = (e / g.E) % g.E, e2 = e / (g.E * g.E);
        T c = T(0);
        for (int nn = 0; nn < n3; ++nn) {
            const int n0 = nn % P1, n1 = (nn / P1) % P1, n2 = nn / (P1 * P1);
            const int x[3] = {e0 * P1 + n0, e1 * P1 + n1, e2 * P1 + n2};
            c += ft.L[q0][n0] * ft.L[q1][n1] * ft.L[q2][n2] * W[(int64_t)e * n3 + nn] * sv[lidx<3>(g, x)];
        }
        cbuf[i] = c;
    }
    __syncthreads();
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
    __syncthreads();
    for (int i = threadIdx.x; i < EE * n3; i += blockDim.x) {
        const int e = i / n3, nn = i % n3;
        const int n0 = nn % P1, n1 = (nn / P1) % P1, n2 = nn / (P1 * P1);
        const int e0 = e % g.E, e1 = (e / g.E) % g.E, e2 = e / (g.E * g.E);
        const T* c = cbuf + e * m3;
        T z = T(0);
        for (int q = 0; q < m3; ++q) {
            const int q0 = q % P, q1 = (q / P) % P, q2 = q / (P * P);
            z += ft.L[q0][n0] * ft.L[q1][n1] * ft.L[q2][n2] * c[q];
        }
        const int x[3] = {e0 * P1 + n0, e1 * P1 + n1, e2 * P1 + n2};
        sv[lidx<3>(g, x)] = z;
    }
    __syncthreads();
}

template <typename T, int P, bool COMP>
__global__ void __launch_bounds__(256) fm_stage_kernel(FmArgs<T> a, Tab<T, P> tb, FmTab<T, P> ft) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    using G = ShapeR<3, P>;
    G g(a.E);
    constexpr int P1 = P + 1;
    T* sF = reinterpret_cast<T*>(smem_raw);   // flux along the current d, padded
    T* sl = sF + g.SS;                        // Laplacian accumulator, then the new v
    T* sc = sl + g.LS;                        // compensation of v (COMP)
    T* cbuf = sc + g.LS;                      // truncation coefficients
    const int mode = a.mode;
    const T* ysrc = (mode == MODE_RHS || mode == MODE_STAGE1) ? a.u : a.y;
    for (int item = blockIdx.x; item < a.nitems; item += gridDim.x) {
        const BlockItem& it = a.items[item];
        const T inv_h = T(1) / T(it.h);
        const double t = stage_time(a.tinfo, it.problem, mode);
        const T* cf = a.coef + (int64_t)item * 10 * g.NN;
        const T* Vb = a.V + (int64_t)item * 3 * g.NN;
        for (int d = 0; d < 3; ++d) {
            const int sd = g.sstride(d), ld = g.lstride(d);
            // F^d = S[d] . V at the owned nodes
            for (int n = threadIdx.x; n < g.NN; n += blockDim.x) {
                int x[3];
                owned_coords<3>(g, n, x);
                T F = T(0);
#pragma unroll
                for (int ci = 0; ci < 3; ++ci) F += cf[(1 + 3 * d + ci) * g.NN + n] * Vb[ci * g.NN + n];
                sF[sidx<3>(g, x)] = F;
            }
            // ... and at the two ghost planes along d, with the face node's S[d]
            for (int i = threadIdx.x; i < 2 * g.F; i += blockDim.x) {
                const int side = i / g.F, tt = i % g.F;
                const int f = 2 * d + side;
                int xo[3], xg[3];
                plane_coords<3>(g, d, tt, side == 0 ? 0 : g.N - 1, xo);
                plane_coords<3>(g, d, tt, side == 0 ? -1 : g.N, xg);
                const int o = oidx<3>(g, xo);
                T Vg[3];
                if (it.nb[f] < 0) {
                    const double* X = a.bnd_x + (int64_t)(it.slot + f) * 3 * g.F;
                    const double th = a.wave.k[0] * X[tt] + a.wave.k[1] * X[g.F + tt] +
                                      a.wave.k[2] * X[2 * g.F + tt] - a.wave.omega * t + a.wave.phi;
                    const double c = cos(th);
#pragma unroll
                    for (int ci = 0; ci < 3; ++ci) Vg[ci] = (T)(a.wave.k[ci] * c);
                } else {
                    const T* src = a.fv + (int64_t)it.nb[f] * 3 * g.F;
                    const int t2 = oriented(tt, g.N, face_orient(it, f));
#pragma unroll
                    for (int ci = 0; ci < 3; ++ci) Vg[ci] = src[ci * g.F + t2];
                }
                T F = T(0);
#pragma unroll
                for (int ci = 0; ci < 3; ++ci) F += cf[(1 + 3 * d + ci) * g.NN + o] * Vg[ci];
                sF[sidx<3>(g, xg)] = F;
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
            const int s = a.eslot[item];
            if (s == 0) {
                truncate_block<T, 3, P, false, 0>(g, tb, sl, nullptr);
                if (final_comp) truncate_block<T, 3, P, false, 0>(g, tb, sc, nullptr);
            } else {
                fm_project_block<T, P>(g, a, ft, s - 1, sl, cbuf);
                if (final_comp) fm_project_block<T, P>(g, a, ft, s - 1, sc, cbuf);
            }
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

// The standalone truncation of the full metric (twoldg_truncate).
template <typename T, int P>
__global__ void __launch_bounds__(256) fm_truncate_kernel(FmArgs<T> a, Tab<T, P> tb, FmTab<T, P> ft) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    using G = ShapeR<3, P>;
    G g(a.E);
    T* sv = reinterpret_cast<T*>(smem_raw);
    T* cbuf = sv + g.LS;
    for (int item = blockIdx.x; item < a.nitems; item += gridDim.x) {
        T* v = a.u + a.items[item].off + g.NN;
        for (int n = threadIdx.x; n < g.NN; n += blockDim.x) {
            int x[3];
            owned_coords<3>(g, n, x);
            sv[lidx<3>(g, x)] = v[n];
        }
        __syncthreads();
        const int s = a.eslot[item];
        if (s == 0) truncate_block<T, 3, P, false, 0>(g, tb, sv, nullptr);
        else fm_project_block<T, P>(g, a, ft, s - 1, sv, cbuf);
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
        double s = block_reduce_sum<3>(local, red);
        if (threadIdx.x == 0) a.partial[item] = 0.5 * s;
        __syncthreads();
    }
}

}  // namespace twoldg
