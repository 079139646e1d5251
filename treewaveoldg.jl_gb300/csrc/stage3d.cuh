// The fused RK stage for 3D blocks with a compile-time shape, one thread per
// (a, b) position of the block's N x N cross-section (N^2 threads).
//
// For every direction d a thread owns the E element lines along d at its
// tangential position (a, b) -- (x1, x2) for d = 0, (x0, x2) for d = 1,
// (x0, x1) for d = 2 -- the two face points (a, b) of the faces normal to d,
// and for the pointwise phases the column (x0, x1) = (a, b), x2 = 0..N-1,
// whose global index is tid + N^2 x2 (coalesced). So every shared-memory and
// global address of the kernel is one of three per-thread bases plus a
// compile-time offset, and every loop unrolls completely. The arithmetic is
// the generic stage's (kernels.cuh: gradient_along, laplacian_along,
// truncate_block, stage_points), applied in the same order, so the results
// are the same bit for bit.
#pragma once

#include "kernels.cuh"

namespace twoldg {

template <typename T, int P, int E>
struct Stage3D {
    static constexpr int P1 = P + 1;
    static constexpr int N = E * P1;
    static constexpr int F = N * N;
    static constexpr int NN = N * F;
    static constexpr int SX = N + 3, SY = N + 2, SXY = SX * SY;  // padded u / gradient
    static constexpr int SS = SXY * SY;
    static constexpr int LX = N + 1, LXY = LX * N;               // ghost-free v
    static constexpr int LS = LXY * N;
    static constexpr int NT = F;
    static constexpr size_t bytes = (2 * (size_t)SS + (size_t)LS) * sizeof(T) + 1024;
    static constexpr int by_smem = (int)((227 * 1024) / bytes);
    static constexpr int by_regs = 65536 / (NT * 64) > 0 ? 65536 / (NT * 64) : 1;
    static constexpr int MINB = by_smem < 1 ? 1 : (by_smem < by_regs ? by_smem : by_regs);
    // this kernel serves shapes whose cross-section fills whole warps
    static constexpr bool usable = F >= 64 && F <= 1024 && F % 32 == 0;
    __host__ __device__ static constexpr int sstride(int d) { return d == 0 ? 1 : d == 1 ? SX : SXY; }
    __host__ __device__ static constexpr int lstride(int d) { return d == 0 ? 1 : d == 1 ? LX : LXY; }
};

template <typename T, int P, int E, bool COMP>
__global__ void __launch_bounds__(Stage3D<T, P, E>::NT, Stage3D<T, P, E>::MINB)
    stage3d_kernel(StageArgs<T> a, Tab<T, P> tb) {
    using S = Stage3D<T, P, E>;
    constexpr int P1 = S::P1, N = S::N, F = S::F, NN = S::NN;
    constexpr int SX = S::SX, SXY = S::SXY, LX = S::LX, LXY = S::LXY;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* su = reinterpret_cast<T*>(smem_raw);
    T* sg = su + S::SS;
    T* sl = sg + S::SS;
    const int tid = threadIdx.x;
    const int ca = tid % N, cb = tid / N;
    // padded index of the node with x_d = 0 on this thread's line along d
    const int sbase[3] = {1 + SX * (ca + 1) + SXY * (cb + 1), (ca + 1) + SX + SXY * (cb + 1),
                          (ca + 1) + SX * (cb + 1) + SXY};
    // ghost-free index of the same nodes
    const int lbase[3] = {LX * ca + LXY * cb, ca + LXY * cb, ca + LX * cb};
    const int mode = a.mode;
    const T* ysrc = (mode == MODE_RHS || mode == MODE_STAGE1) ? a.u : a.y;

    for (int item = blockIdx.x; item < a.nitems; item += gridDim.x) {
        const BlockItem& it = a.items[item];
        const T inv_h = T(1) / T(it.h);
        const T* yu = ysrc + it.off;
        // u of the block: the column (ca, cb), x2 = 0..N-1
#pragma unroll
        for (int j = 0; j < N; ++j) su[sbase[2] + SXY * j] = yu[tid + F * j];
        // u ghosts: face point (ca, cb) of each face
#pragma unroll
        for (int f = 0; f < 6; ++f) {
            const int d = f >> 1, side = f & 1;
            T v;
            if (it.flags & (1u << f)) v = a.ugd[(int64_t)(it.slot + f) * F + tid];
            else v = a.fu_in[(int64_t)it.nb[f] * F + tid];
            su[sbase[d] + (side ? N : -1) * S::sstride(d)] = v;
        }
        __syncthreads();
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const int sd = S::sstride(d), ld = S::lstride(d);
            // gradient along d on the thread's E lines, scaled by 1/h
#pragma unroll
            for (int e = 0; e < E; ++e) {
                const int base = sbase[d] + e * P1 * sd;
                T w[P + 3], out[P + 1];
#pragma unroll
                for (int k = 0; k < P + 3; ++k) w[k] = su[base + (k - 1) * sd];
                line_derivative<T, P>(tb, w, out);
#pragma unroll
                for (int i = 0; i <= P; ++i) sg[base + i * sd] = out[i] * inv_h;
            }
            // the two gradient ghosts at (ca, cb)
#pragma unroll
            for (int side = 0; side < 2; ++side) {
                const int f = 2 * d + side;
                T v;
                if (it.flags & (1u << f)) {
                    v = a.ggd[(int64_t)(it.slot + f) * F + tid];
                } else {
                    const int nslot = it.nb[f];
                    const T own = su[sbase[d] + (side ? N - 1 : 0) * sd];
                    const T gnb = (a.fog_in[(int64_t)nslot * F + tid] + ghost_coef<T, P>(tb, nslot & 1) * own) * inv_h;
                    v = (it.flags & (1u << (8 + f))) ? -gnb : gnb;
                }
                sg[sbase[d] + (side ? N : -1) * sd] = v;
            }
            __syncthreads();
            // Laplacian term along d
#pragma unroll
            for (int e = 0; e < E; ++e) {
                const int base = sbase[d] + e * P1 * sd;
                const int lb = lbase[d] + e * P1 * ld;
                T w[P + 3], out[P + 1];
#pragma unroll
                for (int k = 0; k < P + 3; ++k) w[k] = sg[base + (k - 1) * sd];
                line_derivative<T, P>(tb, w, out);
#pragma unroll
                for (int i = 0; i <= P; ++i) {
                    if (d == 0) sl[lb + i * ld] = out[i];
                    else sl[lb + i * ld] += out[i];
                }
            }
            __syncthreads();
        }
        const T* yv = ysrc + it.off + NN;
        if (mode == MODE_RHS) {
            T* du = a.du + it.off;
#pragma unroll
            for (int j = 0; j < N; ++j) {
                du[tid + F * j] = yv[tid + F * j];
                du[NN + tid + F * j] = sl[lbase[2] + LXY * j] * inv_h;
            }
            __syncthreads();
            continue;
        }
        const RkCoef<T> rc(mode, a.dts[it.problem]);
        const T* __restrict__ un = a.u + it.off;
        T* __restrict__ acc = a.acc + it.off;
        T* __restrict__ comp = COMP ? a.comp + it.off : nullptr;
        T* sc = sg;  // compensation of v during the final truncation (ghost-free layout)
        constexpr int B = 4;
#pragma unroll
        for (int j0 = 0; j0 < N; j0 += B) {
            T y[B], uu[B], uv[B], au[B], av[B], cu[B], cvi[B];
#pragma unroll
            for (int q = 0; q < B; ++q) {
                if (j0 + q < N) {
                    const int n = tid + F * (j0 + q);
                    y[q] = yv[n];
                    uu[q] = un[n];
                    uv[q] = un[NN + n];
                    if (mode != 1) {
                        au[q] = acc[n];
                        av[q] = acc[NN + n];
                    }
                    if (COMP && mode == MODE_STAGE4) {
                        cu[q] = comp[n];
                        cvi[q] = comp[NN + n];
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < B; ++q) {
                if (j0 + q < N) {
                    const int j = j0 + q;
                    const int n = tid + F * j;
                    const int s0 = sbase[2] + SXY * j, l0 = lbase[2] + LXY * j;
                    T lap[1] = {sl[l0]};
                    T nu[1], nv[1], cv[1];
                    T yq[1] = {y[q]}, uuq[1] = {uu[q]}, uvq[1] = {uv[q]}, auq[1] = {au[q]}, avq[1] = {av[q]},
                      cuq[1] = {cu[q]}, cviq[1] = {cvi[q]};
                    stage_points<T, COMP, 1>(mode, rc, yq, uuq, uvq, auq, avq, cuq, cviq, lap, inv_h, nu, nv, cv);
                    if (mode != MODE_STAGE4) {
                        acc[n] = auq[0];
                        acc[NN + n] = avq[0];
                    }
                    if (COMP && mode == MODE_STAGE4) comp[n] = cuq[0];
                    su[s0] = nu[0];
                    sl[l0] = nv[0];
                    if (COMP && mode == MODE_STAGE4) sc[l0] = cv[0];
                }
            }
        }
        __syncthreads();
        const bool final_comp = COMP && mode == MODE_STAGE4;
        if (a.truncate) {
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const int ld = S::lstride(d);
#pragma unroll
                for (int e = 0; e < E; ++e) {
                    const int lb = lbase[d] + e * P1 * ld;
                    T v[P1];
                    T c = T(0);
#pragma unroll
                    for (int jj = 0; jj < P1; ++jj) { v[jj] = sl[lb + jj * ld]; c += tb.td[jj] * v[jj]; }
                    if (final_comp) {
                        T cc = T(0);
#pragma unroll
                        for (int jj = 0; jj < P1; ++jj) cc += tb.td[jj] * sc[lb + jj * ld];
                        c += cc;
#pragma unroll
                        for (int i = 0; i < P1; ++i) {
                            T s, err;
                            two_sum(v[i], -(tb.tm[i] * c), s, err);
                            sl[lb + i * ld] = s;
                            sc[lb + i * ld] += err;
                        }
                    } else {
#pragma unroll
                        for (int i = 0; i < P1; ++i) sl[lb + i * ld] = v[i] - tb.tm[i] * c;
                    }
                }
                __syncthreads();
            }
        }
        T* out = (mode == MODE_STAGE4 ? a.u : a.y) + it.off;
#pragma unroll
        for (int j = 0; j < N; ++j) {
            out[tid + F * j] = su[sbase[2] + SXY * j];
            out[NN + tid + F * j] = sl[lbase[2] + LXY * j];
            if (final_comp) comp[NN + tid + F * j] = sc[lbase[2] + LXY * j];
        }
        // face export of the new u at (ca, cb)
#pragma unroll
        for (int f = 0; f < 6; ++f) {
            const int d = f >> 1, side = f & 1;
            const int sd = S::sstride(d);
            const int base = sbase[d] + (side ? N - 1 - P : 0) * sd;
            T e[P + 1];
#pragma unroll
            for (int k = 0; k <= P; ++k) e[k] = su[base + k * sd];
            const int64_t o = (int64_t)(it.slot + f) * F + tid;
            a.fu_out[o] = side == 0 ? e[0] : e[P];
            a.fog_out[o] = own_face_part<T, P>(tb, side, e);
        }
        __syncthreads();
    }
}

}  // namespace twoldg
