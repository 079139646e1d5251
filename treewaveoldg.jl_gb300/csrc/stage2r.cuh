// The fused RK stage for 2D blocks with a compile-time shape, whole element
// lines in registers: the two-dimensional counterpart of stage3r.cuh. One
// thread per y-column of a block (N threads), K = 128 / N blocks per CTA, so
// that the small blocks of a 2D forest (N = 6 to 24 nodes a side) still fill
// a CTA. A thread loads its column straight into registers and forms the y
// gradient (with its two ghosts) and the y Laplacian term there; the x lines
// (thread c takes row c) read u from a padded shared copy and add their
// Laplacian term into the shared accumulator. The RK combination runs element
// by element down the column with the y truncation in registers; the x
// truncation follows in shared memory. Three barriers a block, against the
// generic kernel's one per phase and dimension.
#pragma once

#include "stage3r.cuh"

namespace twoldg {

template <typename T, int P, int E, bool COMP>
struct Stage2R {
    static constexpr int P1 = P + 1;
    static constexpr int N = E * P1;
    static constexpr int NN = N * N;
    static constexpr int K = 128 / N > 0 ? 128 / N : 1;   // blocks per CTA
    static constexpr int NT = K * N;
    // u rows with the two x ghosts, and the accumulator / new v rows, each
    // thread's row read and written as whole 16-byte words: NU and NL words
    // a row, at pitches of an odd number of 16-byte words, so that the rows
    // a quarter-warp walks fall in distinct banks
    static constexpr int VW = 16 / sizeof(T);
    static constexpr int NU = (N + 2 + VW - 1) / VW, NL = (N + VW - 1) / VW;
    static constexpr int SX = vec_pitch<T>(N + 3), LX = vec_pitch<T>(N);
    static_assert(SX >= NU * VW && LX >= NL * VW, "a row's last 16-byte word stays in its pitch");
    static constexpr int SS = SX * N, LS = LX * N;
    static constexpr int PER = SS + LS + (COMP ? LS : 0);   // words of one block
    static constexpr size_t words = (size_t)K * PER;
    static constexpr bool usable = N <= 32;
};

// A thread's row of NV 16-byte words at p (16-byte aligned) to and from
// registers.
template <typename T, int NV>
__device__ __forceinline__ void row_load(const T* p, T (&r)[NV * (16 / sizeof(T))]) {
    using V = typename V16<T>::type;
    constexpr int VW = 16 / sizeof(T);
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        const V t = reinterpret_cast<const V*>(p)[k];
        const T* e = reinterpret_cast<const T*>(&t);
#pragma unroll
        for (int q = 0; q < VW; ++q) r[k * VW + q] = e[q];
    }
}

template <typename T, int NV>
__device__ __forceinline__ void row_store(T* p, const T (&r)[NV * (16 / sizeof(T))]) {
    using V = typename V16<T>::type;
    constexpr int VW = 16 / sizeof(T);
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        V t;
        T* e = reinterpret_cast<T*>(&t);
#pragma unroll
        for (int q = 0; q < VW; ++q) e[q] = r[k * VW + q];
        reinterpret_cast<V*>(p)[k] = t;
    }
}

// The truncation of the E element lines of a thread's contiguous row (the
// accumulator row sl and, in stage 4, the compensation row sc), each read
// and written as whole 16-byte words; the arithmetic of truncate_lines.
template <typename T, int P, int E, int NV>
__device__ __forceinline__ void truncate_row(const Tab<T, P>& tb, T* sl, T* sc, bool final_comp) {
    constexpr int P1 = P + 1, VW = 16 / sizeof(T);
    T v[NV * VW];
    row_load<T, NV>(sl, v);
    if (final_comp) {
        T w[NV * VW];
        row_load<T, NV>(sc, w);
#pragma unroll
        for (int e = 0; e < E; ++e) {
            T c = T(0);
#pragma unroll
            for (int q = 0; q < P1; ++q) c += tb.td[q] * v[e * P1 + q];
            T cc = T(0);
#pragma unroll
            for (int q = 0; q < P1; ++q) cc += tb.td[q] * w[e * P1 + q];
            c += cc;
#pragma unroll
            for (int q = 0; q < P1; ++q) {
                T s, err;
                two_sum(v[e * P1 + q], -(tb.tm[q] * c), s, err);
                v[e * P1 + q] = s;
                w[e * P1 + q] += err;
            }
        }
        row_store<T, NV>(sc, w);
    } else {
#pragma unroll
        for (int e = 0; e < E; ++e) {
            T c = T(0);
#pragma unroll
            for (int q = 0; q < P1; ++q) c += tb.td[q] * v[e * P1 + q];
#pragma unroll
            for (int q = 0; q < P1; ++q) v[e * P1 + q] = v[e * P1 + q] - tb.tm[q] * c;
        }
    }
    row_store<T, NV>(sl, v);
}

// FM: the stage the instantiation runs (1-4), so that each stage's code holds
// only its own data flow, or 0 for the mode in the arguments.
template <typename T, int P, int E, bool COMP, int FM = 0>
__global__ void __launch_bounds__(Stage2R<T, P, E, COMP>::NT)
    stage2r_kernel(StageArgs<T> a, Tab<T, P> tb) {
    using S = Stage2R<T, P, E, COMP>;
    constexpr int P1 = S::P1, N = S::N, NN = S::NN, SX = S::SX, LX = S::LX, K = S::K, VW = S::VW;
    constexpr int NU = S::NU, NL = S::NL;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int bs = threadIdx.x / N, c = threadIdx.x % N;   // block slot of the CTA, column
    T* su = reinterpret_cast<T*>(smem_raw) + bs * S::PER;
    T* sl = su + S::SS;
    T* sc = sl + S::LS;   // compensated only
    const int mode = FM ? FM : a.mode;
    // the stages' data flow is the 3D kernel's: stage 1 stores only the
    // truncated v-rate k1_v in the v half of `y`, stage 2 forms Y2 and the
    // first increment from u^n and k1_v
    const T* ysrc = (mode == MODE_RHS || mode == MODE_STAGE1 || mode == 2) ? a.u : a.y;
    const T* vsrc = mode == 2 ? a.y : ysrc;
    const bool final_comp = COMP && mode == MODE_STAGE4;

    // the first blocks' operands are asked into L2 (a hint) before the wait
    // on the previous stage, as in the 3D kernel
    const int first = blockIdx.x * K + bs;
    if (c == 0 && first < a.nitems) prefetch_stage3r<T>(a, first, NN, (int)gridDim.x * K);
    grid_dependency_wait();
    if (a.release) grid_dependents_launch();
    for (int base = blockIdx.x * K; base < a.nitems; base += gridDim.x * K) {
        const int item = base + bs;
        // every thread passes every barrier; a slot past the last item holds
        // no block and touches no memory
        const bool live = item < a.nitems;
        const BlockItem* it = live ? &a.items[item] : nullptr;
        // the two passes differentiate without 1/h; the Laplacian takes 1/h^2
        T hb = T(0), inv_h2 = T(0);
        uint32_t flags = 0;
        int slot = 0, nb[4] = {0, 0, 0, 0};
        T ug[4], gp[4];
        if (live) {
            // the block's stage operands (and the next block this slot takes)
            // into L2 while the CTA computes
            if (c == 0 && item != first) prefetch_stage3r<T>(a, item, NN, (int)gridDim.x * K);
            flags = it->flags;
            slot = it->slot;
#pragma unroll
            for (int f = 0; f < 4; ++f) nb[f] = it->nb[f];
            hb = T(it->h);
            const T inv_h = T(1) / hb;
            inv_h2 = inv_h * inv_h;
            const T* yu = ysrc + it->off;
            T line[N + 2];
            if (mode == 2) {
                const T cn1 = a.rk[4 * it->problem + 2];
#pragma unroll
                for (int j = 0; j < N; ++j) line[1 + j] = yu[c + N * j] + cn1 * yu[NN + c + N * j];
            } else {
#pragma unroll
                for (int j = 0; j < N; ++j) line[1 + j] = yu[c + N * j];
            }
            // face f's ghosts at this thread's tangential point: x faces at
            // row x1 = c, y faces at column x0 = c
#pragma unroll
            for (int f = 0; f < 4; ++f) {
                if (flags & (1u << f)) {
                    ug[f] = a.ugd[(int64_t)(slot + f) * N + c];
                    gp[f] = a.ggd[(int64_t)(slot + f) * N + c];
                } else {
                    ug[f] = a.fu_in[(int64_t)nb[f] * N + c];
                    gp[f] = a.fog_in[(int64_t)nb[f] * N + c];
                }
            }
#pragma unroll
            for (int j = 0; j < N; ++j) su[j * SX + c + 1] = line[1 + j];
            su[c * SX] = ug[0];
            su[c * SX + N + 1] = ug[1];
            line[0] = ug[2];
            line[N + 1] = ug[3];
            // ---- y: the column in registers
            T g[N + 2], gi[N], lap[N];
            line_full<T, P, E>(tb, line, gi, T(1));
#pragma unroll
            for (int j = 0; j < N; ++j) g[1 + j] = gi[j];
            g[0] = grad_ghost_raw<T, P>(tb, flags, nb[2], 2, gp[2], line[1], hb);
            g[N + 1] = grad_ghost_raw<T, P>(tb, flags, nb[3], 3, gp[3], line[N], hb);
            line_full<T, P, E>(tb, g, lap, T(1));
#pragma unroll
            for (int j = 0; j < N; ++j) sl[j * LX + c] = lap[j];
        }
        __syncthreads();
        // ---- x: row c from the shared copy of u
        if (live) {
            T row[NU * VW], line[N + 2], g[N + 2], gi[N], lap[N];
            row_load<T, NU>(su + c * SX, row);
#pragma unroll
            for (int k = 0; k < N + 2; ++k) line[k] = row[k];
            line_full<T, P, E>(tb, line, gi, T(1));
#pragma unroll
            for (int j = 0; j < N; ++j) g[1 + j] = gi[j];
            g[0] = grad_ghost_raw<T, P>(tb, flags, nb[0], 0, gp[0], line[1], hb);
            g[N + 1] = grad_ghost_raw<T, P>(tb, flags, nb[1], 1, gp[1], line[N], hb);
            line_full<T, P, E>(tb, g, lap, T(1));
            T acc_row[NL * VW];
            row_load<T, NL>(sl + c * LX, acc_row);
#pragma unroll
            for (int i = 0; i < N; ++i) acc_row[i] += lap[i];
            row_store<T, NL>(sl + c * LX, acc_row);
        }
        __syncthreads();
        if (mode == MODE_RHS) {
            if (live) {
                const T* yv = ysrc + it->off + NN;
                T* du = a.du + it->off;
#pragma unroll
                for (int j = 0; j < N; ++j) {
                    du[c + N * j] = yv[c + N * j];
                    du[NN + c + N * j] = sl[j * LX + c] * inv_h2;
                }
            }
            __syncthreads();
            continue;
        }
        // ---- the RK combination down the column, element by element, with
        // the truncation along y in registers
        if (live) {
            const T* yv = vsrc + it->off + NN;
            const RkCoef<T> rc(mode, a.rk + 4 * it->problem);
            const RkCoef<T> rc1(1, a.rk + 4 * it->problem);   // dt/6 and dt/2
            const T* __restrict__ un = a.u + it->off;
            T* __restrict__ acc = a.acc + it->off;
            T* __restrict__ comp = COMP ? a.comp + it->off : nullptr;
            T* out = (mode == MODE_STAGE4 ? a.u : a.y) + it->off;
#pragma unroll
            for (int ey = 0; ey < E; ++ey) {
                T y[P1], uu[P1], uv[P1], au[P1], av[P1], cu[P1], cvi[P1];
#pragma unroll
                for (int q = 0; q < P1; ++q) {
                    const int n = c + N * (ey * P1 + q);
                    y[q] = yv[n];
                    if (mode == MODE_STAGE1) {
                        uu[q] = su[(ey * P1 + q) * SX + c + 1];
                        uv[q] = y[q];
                    } else {
                        uu[q] = un[n];
                        uv[q] = un[NN + n];
                    }
                    if (mode == 2) {
                        // y[q] holds k1_v: Y2's v and the first increment
                        const T k1v = y[q];
                        y[q] = uv[q] + rc1.cn * k1v;
                        au[q] = rc1.ca * uv[q];
                        av[q] = rc1.ca * k1v;
                    } else if (mode != MODE_STAGE1) {
                        au[q] = acc[n];
                        av[q] = acc[NN + n];
                    }
                    if (final_comp) {
                        cu[q] = comp[n];
                        cvi[q] = comp[NN + n];
                    }
                }
                T nu[P1], nv[P1], cv[P1];
#pragma unroll
                for (int q = 0; q < P1; ++q) {
                    const int j = ey * P1 + q;
                    T lap[1] = {sl[j * LX + c]};
                    T o_u[1], o_v[1], o_c[1];
                    T yq[1] = {y[q]}, uuq[1] = {uu[q]}, uvq[1] = {uv[q]}, auq[1] = {au[q]}, avq[1] = {av[q]},
                      cuq[1] = {cu[q]}, cviq[1] = {cvi[q]};
                    if (mode == MODE_STAGE1) {
                        // Y2's u for the face export; the v-rate, truncated below and stored
                        o_u[0] = uuq[0] + rc.cn * yq[0];
                        o_v[0] = lap[0] * inv_h2;
                        o_c[0] = T(0);
                    } else {
                        stage_points<T, COMP, 1>(mode, rc, yq, uuq, uvq, auq, avq, cuq, cviq, lap, inv_h2, o_u,
                                                 o_v, o_c);
                    }
                    au[q] = auq[0];
                    av[q] = avq[0];
                    cu[q] = cuq[0];
                    nu[q] = o_u[0];
                    nv[q] = o_v[0];
                    cv[q] = o_c[0];
                }
                if (a.truncate) {
                    T cc0 = T(0);
#pragma unroll
                    for (int q = 0; q < P1; ++q) cc0 += tb.td[q] * nv[q];
                    if (final_comp) {
                        T cc = T(0);
#pragma unroll
                        for (int q = 0; q < P1; ++q) cc += tb.td[q] * cv[q];
                        cc0 += cc;
#pragma unroll
                        for (int q = 0; q < P1; ++q) {
                            T s, err;
                            two_sum(nv[q], -(tb.tm[q] * cc0), s, err);
                            nv[q] = s;
                            cv[q] += err;
                        }
                    } else {
#pragma unroll
                        for (int q = 0; q < P1; ++q) nv[q] = nv[q] - tb.tm[q] * cc0;
                    }
                }
#pragma unroll
                for (int q = 0; q < P1; ++q) {
                    const int j = ey * P1 + q;
                    const int n = c + N * j;
                    if (mode == 2 || mode == 3) {
                        acc[n] = au[q];
                        acc[NN + n] = av[q];
                        out[n] = nu[q];
                    }
                    if (final_comp) comp[n] = cu[q];
                    su[j * SX + c + 1] = nu[q];
                    sl[j * LX + c] = nv[q];
                    if (final_comp) sc[j * LX + c] = cv[q];
                }
                // the column's own y faces from its first and last element
                if (ey == 0 || ey == E - 1) {
                    const int side = ey == 0 ? 0 : 1;
                    const int64_t o = (int64_t)(slot + 2 + side) * N + c;
                    a.fu_out[o] = side == 0 ? nu[0] : nu[P];
                    a.fog_out[o] = own_face_part<T, P>(tb, side, nu);
                }
            }
        }
        __syncthreads();
        // ---- the x faces of the new u (row c), and the truncation along x
        if (live) {
            T row[NU * VW];
            row_load<T, NU>(su + c * SX, row);
#pragma unroll
            for (int side = 0; side < 2; ++side) {
                T e[P1];
#pragma unroll
                for (int k = 0; k < P1; ++k) e[k] = row[1 + (side ? N - P1 : 0) + k];
                const int64_t o = (int64_t)(slot + side) * N + c;
                a.fu_out[o] = side == 0 ? e[0] : e[P];
                a.fog_out[o] = own_face_part<T, P>(tb, side, e);
            }
            if (a.truncate) truncate_row<T, P, E, NL>(tb, sl + c * LX, sc + c * LX, final_comp);
        }
        __syncthreads();
        // ---- the new v of the column (and in stage 4 its u)
        if (live) {
            T* out = (mode == MODE_STAGE4 ? a.u : a.y) + it->off;
            T* __restrict__ comp = COMP ? a.comp + it->off : nullptr;
#pragma unroll
            for (int j = 0; j < N; ++j) {
                if (mode == MODE_STAGE4) out[c + N * j] = su[j * SX + c + 1];
                out[NN + c + N * j] = sl[j * LX + c];
                if (final_comp) comp[NN + c + N * j] = sc[j * LX + c];
            }
        }
        __syncthreads();
    }
}

}  // namespace twoldg
