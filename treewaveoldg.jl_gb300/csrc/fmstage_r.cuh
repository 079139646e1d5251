// The full-metric stage pass with a compile-time block shape: the kernel,
// its attributes and its launches (declared in fullmetric.cuh). Only the
// ball problems run it, so it lives in translation units of its own
// (kernels_d3_p<P>_fm.cu), which the build compiles beside the others.
#pragma once
#include "fullmetric.cuh"

namespace twoldg {

// The stage pass with a compile-time block shape (E = 2 or 4), in the
// register-line layout of stage3r_kernel: one thread per (a, b) position of
// the block's cross-section. D_z F^z comes from the thread's own column of
// F^z in registers with its two ghost fluxes; F^x and then F^y go through one
// padded shared array, whose x and y lines give D_x F^x into the accumulator
// and D_y F^y added to it; the RK combination runs down the column with D_z
// F^z from registers. The truncation, the new v's store and u's face export
// are the run-time-shape kernel's, on the same ghost-free accumulator layout.
template <typename T, int P, int E, bool COMP>
struct FmStageR {
    using S = Stage3R<T, P, E, false>;
    static constexpr int N = S::N, LXg = N + 1;
    static constexpr size_t LSg = (size_t)LXg * N * N;   // the run-time-shape kernel's accumulator
    static constexpr size_t cbuf = (size_t)E * E * E * (P + 1) * P * P;
    static constexpr size_t words = (size_t)S::SS + (COMP ? 2 : 1) * LSg + cbuf;
    // CTAs an SM holds: by shared memory, and by 80 registers a thread
    static constexpr int by_smem = (int)((227 * 1024) / (words * sizeof(T) + 1024));
    static constexpr int by_regs = 65536 / (S::NT * 80) > 0 ? 65536 / (S::NT * 80) : 1;
    static constexpr int MINB = by_smem < 1 ? 1 : (by_smem < by_regs ? by_smem : by_regs);
};

template <typename T, int P, int E, bool COMP, int FM>
__global__ void __launch_bounds__(Stage3R<T, P, E, false>::NT, (FmStageR<T, P, E, COMP>::MINB))
    fm_stage_r_kernel(FmArgs<T> a, Tab<T, P> tb, FmTab<T, P> ft) {
    using S = Stage3R<T, P, E, false>;
    using R = FmStageR<T, P, E, COMP>;
    constexpr int N = S::N, F = S::F, NN = S::NN, VW = S::VW;
    constexpr int SX = S::SX, SXY = S::SXY, LX = R::LXg, LP = LX * N;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sF = reinterpret_cast<T*>(smem_raw);   // F^x, then F^y, padded
    T* sl = sF + S::SS;                       // the accumulator, then the new v (LX = N + 1)
    T* sc = sl + R::LSg;                      // compensation of v (COMP)
    T* cbuf = sl + (COMP ? 2 : 1) * R::LSg;   // truncation coefficients
    __shared__ T sLeg[P * (P + 1)];
    stage_legendre<T, P>(ft, sLeg);
    using G = ShapeR<3, P>;
    G g(E);
    const int tid = threadIdx.x, ca = tid % N, cb = tid / N;
    const int s0 = 1 + SX * (ca + 1) + SXY * cb;   // x-line (x1, x2) = (ca, cb)
    const int s1 = (ca + 1) + SX + SXY * cb;       // y-line (x0, x2) = (ca, cb)
    const int s2 = (ca + 1) + SX * (cb + 1);       // z column (x0, x1) = (ca, cb)
    const int mode = FM;
    const T* ysrc = (mode == MODE_STAGE1) ? a.u : a.y;
    // a block's operands into L2 (a hint): the fluxes, sqrt(g), the stage
    // operands and the block's projection tables
    auto prefetch = [&](int item) {
        const int64_t off = a.items[item].off;
        const size_t b = (size_t)NN * sizeof(T);
        prefetch_l2(a.V + (int64_t)item * 3 * NN, 3 * b);
        prefetch_l2(a.coef + (int64_t)item * 10 * NN, b);
        prefetch_l2(ysrc + off, 2 * b);
        if (mode != MODE_STAGE1) {
            prefetch_l2(a.u + off, 2 * b);
            prefetch_l2(a.acc + off, 2 * b);
            if (COMP && mode == MODE_STAGE4) prefetch_l2(a.comp + off, 2 * b);
        }
        const int es = a.eslot[item];
        if (a.truncate && es > 0) {
            constexpr int n3 = (P + 1) * (P + 1) * (P + 1), m3 = P * P * P;
            constexpr size_t EE = (size_t)E * E * E;
            prefetch_l2(a.ew + (int64_t)(es - 1) * n3 * EE, n3 * EE * sizeof(T));
            prefetch_l2(a.echol + (int64_t)(es - 1) * m3 * m3 * EE, (size_t)m3 * m3 * EE * sizeof(T));
        }
    };
    // the first block's before the wait on the gradient pass, as in the flat
    // stage kernel (L2 is where that pass's writes land: nothing stale is read)
    if (tid == 0 && (int)blockIdx.x < a.nitems) prefetch(blockIdx.x);
    grid_dependency_wait();
    if (a.release) grid_dependents_launch();
    for (int item = blockIdx.x; item < a.nitems; item += gridDim.x) {
        const BlockItem& it = a.items[item];
        const T inv_h = T(1) / T(it.h);
        const double t = stage_time(a.tinfo, it.problem, mode);
        const T* cf = a.coef + (int64_t)item * 10 * NN;
        const T* Fb = a.V + (int64_t)item * 3 * NN;
        if (tid == 0 && item != (int)blockIdx.x) prefetch(item);
        // D_z F^z down the column, in registers
        T lapz[N];
        {
            T line[N + 2];
#pragma unroll
            for (int j = 0; j < N; ++j) line[1 + j] = Fb[2 * NN + tid + F * j];
            line[0] = fm_flux_ghost(a, it, 4, 2, 0, tid, tid, F, N, NN, t, cf, Fb, ysrc);
            line[N + 1] = fm_flux_ghost(a, it, 5, 2, 1, tid, tid + F * (N - 1), F, N, NN, t, cf, Fb, ysrc);
            line_full<T, P, E>(tb, line, lapz, T(1));
        }
        // D_x F^x: the column's F^x into the padded array, the x line's ghosts
#pragma unroll
        for (int j = 0; j < N; ++j) sF[s2 + SXY * j] = Fb[tid + F * j];
        sF[s0 - 1] = fm_flux_ghost(a, it, 0, 0, 0, tid, N * ca + F * cb, F, N, NN, t, cf, Fb, ysrc);
        sF[s0 + N] = fm_flux_ghost(a, it, 1, 0, 1, tid, (N - 1) + N * ca + F * cb, F, N, NN, t, cf, Fb, ysrc);
        __syncthreads();
        {
            using V = typename V16<T>::type;
            T xl[N + 2], dx[N];
#pragma unroll
            for (int k = 0; k + VW <= N + 2; k += VW) {
                const V v = *reinterpret_cast<const V*>(sF + s0 - 1 + k);
                const T* e = reinterpret_cast<const T*>(&v);
#pragma unroll
                for (int q = 0; q < VW; ++q) xl[k + q] = e[q];
            }
#pragma unroll
            for (int k = (N + 2) / VW * VW; k < N + 2; ++k) xl[k] = sF[s0 - 1 + k];
            line_full<T, P, E>(tb, xl, dx, T(1));
#pragma unroll
            for (int i = 0; i < N; ++i) sl[i + LX * ca + LP * cb] = dx[i];
        }
        __syncthreads();
        // D_y F^y added: the column's F^y over F^x, the y line's ghosts
#pragma unroll
        for (int j = 0; j < N; ++j) sF[s2 + SXY * j] = Fb[NN + tid + F * j];
        sF[s1 - SX] = fm_flux_ghost(a, it, 2, 1, 0, tid, ca + F * cb, F, N, NN, t, cf, Fb, ysrc);
        sF[s1 + N * SX] = fm_flux_ghost(a, it, 3, 1, 1, tid, ca + N * (N - 1) + F * cb, F, N, NN, t, cf, Fb, ysrc);
        __syncthreads();
        {
            T yl[N + 2], dy[N];
#pragma unroll
            for (int k = 0; k < N + 2; ++k) yl[k] = sF[s1 + (k - 1) * SX];
            line_full<T, P, E>(tb, yl, dy, T(1));
#pragma unroll
            for (int i = 0; i < N; ++i) sl[ca + LX * i + LP * cb] += dy[i];
        }
        __syncthreads();
        // the RK combination down the column
        const RkCoef<T> rc(mode, a.rk + 4 * it.problem);
        const T* yv = ysrc + it.off + NN;
        const T* un = a.u + it.off;
        T* acc = a.acc + it.off;
        T* comp = COMP ? a.comp + it.off : nullptr;
        const bool final_comp = COMP && mode == MODE_STAGE4;
        T* out = (mode == MODE_STAGE4 ? a.u : a.y) + it.off;
#pragma unroll 4
        for (int j = 0; j < N; ++j) {
            const int n = tid + F * j, l = ca + LX * cb + LP * j;
            T lap[1] = {(sl[l] + lapz[j]) / cf[n]};
            T yq[1] = {yv[n]}, uuq[1] = {un[n]}, uvq[1] = {un[NN + n]}, auq[1], avq[1], cuq[1], cviq[1];
            if (mode != 1) { auq[0] = acc[n]; avq[0] = acc[NN + n]; }
            if (final_comp) { cuq[0] = comp[n]; cviq[0] = comp[NN + n]; }
            T nu[1], nv[1], cv[1];
            stage_points<T, COMP, 1>(mode, rc, yq, uuq, uvq, auq, avq, cuq, cviq, lap, inv_h, nu, nv, cv);
            if (mode != MODE_STAGE4) { acc[n] = auq[0]; acc[NN + n] = avq[0]; }
            if (final_comp) { comp[n] = cuq[0]; sc[l] = cv[0]; }
            out[n] = nu[0];
            sl[l] = nv[0];
        }
        __syncthreads();
        if (a.truncate) {
            fm_truncate_block<T, P>(g, a, tb, sLeg, item, sl, cbuf);
            if (final_comp) fm_truncate_block<T, P>(g, a, tb, sLeg, item, sc, cbuf);
        }
#pragma unroll 4
        for (int j = 0; j < N; ++j) {
            const int n = tid + F * j, l = ca + LX * cb + LP * j;
            out[NN + n] = sl[l];
            if (final_comp) comp[NN + n] = sc[l];
        }
        // u's face nodes of the new stage value for the next gradient pass
        // (the x and y faces' nodes written by other columns: after the
        // barrier, global writes of the CTA are visible to it)
        __syncthreads();
#pragma unroll
        for (int f = 0; f < 6; ++f) {
            const int side = f & 1;
            int n;
            if (f < 2) n = (side ? N - 1 : 0) + N * ca + F * cb;
            else if (f < 4) n = ca + N * (side ? N - 1 : 0) + F * cb;
            else n = tid + F * (side ? N - 1 : 0);
            a.fu_out[(int64_t)(it.slot + f) * F + tid] = out[n];
        }
        __syncthreads();
    }
}

template <typename K>
inline void fm_stage_r_attr(K kern, int max_smem) {
    cudaFuncAttributes fa{};
    cudaFuncGetAttributes(&fa, kern);
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem - (int)fa.sharedSizeBytes);
    cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
}

template <typename T, int P, int E, bool COMP>
void fm_stage_r_attrs(int max_smem) {
    if constexpr (Stage3R<T, P, E, false>::usable) {
        fm_stage_r_attr(fm_stage_r_kernel<T, P, E, COMP, 1>, max_smem);
        fm_stage_r_attr(fm_stage_r_kernel<T, P, E, COMP, 2>, max_smem);
        fm_stage_r_attr(fm_stage_r_kernel<T, P, E, COMP, 3>, max_smem);
        fm_stage_r_attr(fm_stage_r_kernel<T, P, E, COMP, 4>, max_smem);
    }
}

template <typename T, int P, int E, bool COMP>
size_t fm_stage_r_smem() {
    return FmStageR<T, P, E, COMP>::words * sizeof(T);
}

template <typename T, int P, int E, bool COMP>
cudaError_t fm_stage_r_launch(const FmArgs<T>& a, const Tab<T, P>& tb, const FmTab<T, P>& ft, int grid, int mode,
                              cudaStream_t s, bool pdl) {
    if constexpr (!Stage3R<T, P, E, false>::usable) {
        return cudaErrorInvalidConfiguration;
    } else {
        constexpr int NT = Stage3R<T, P, E, false>::NT;
        const size_t smem = fm_stage_r_smem<T, P, E, COMP>();
        auto go = [&](auto kern) {
            FmArgs<T> b = a;
            b.release = pdl && release_early(kern, grid, NT, smem);
            return launch_kernel(kern, grid, NT, smem, s, pdl, b, tb, ft);
        };
        if (mode == MODE_STAGE1) go(fm_stage_r_kernel<T, P, E, COMP, 1>);
        else if (mode == 2) go(fm_stage_r_kernel<T, P, E, COMP, 2>);
        else if (mode == 3) go(fm_stage_r_kernel<T, P, E, COMP, 3>);
        else if (mode == MODE_STAGE4) go(fm_stage_r_kernel<T, P, E, COMP, 4>);
        else return cudaErrorInvalidValue;
        return cudaGetLastError();
    }
}

// The instantiations of one order: FP64, FP32 and FP32 compensated, E = 2, 4.
#define TWOLDG_FMSTAGE_R_E(T, P, E, COMP)                                                                        \
    template void fm_stage_r_attrs<T, P, E, COMP>(int);                                                          \
    template size_t fm_stage_r_smem<T, P, E, COMP>();                                                            \
    template cudaError_t fm_stage_r_launch<T, P, E, COMP>(const FmArgs<T>&, const Tab<T, P>&, const FmTab<T, P>&, \
                                                           int, int, cudaStream_t, bool);
#define TWOLDG_FMSTAGE_R(P)                  \
    TWOLDG_FMSTAGE_R_E(double, P, 2, false) \
    TWOLDG_FMSTAGE_R_E(double, P, 4, false) \
    TWOLDG_FMSTAGE_R_E(float, P, 2, false)  \
    TWOLDG_FMSTAGE_R_E(float, P, 4, false)  \
    TWOLDG_FMSTAGE_R_E(float, P, 2, true)   \
    TWOLDG_FMSTAGE_R_E(float, P, 4, true)

}  // namespace twoldg
