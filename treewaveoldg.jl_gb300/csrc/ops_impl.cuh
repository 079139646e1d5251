// The templated Ops implementation: fills the constant tables once and
// launches the kernels of kernels.cuh with them.
#pragma once
#include <algorithm>
#include <cmath>

#include "kernels.cuh"
#include "ops.h"
#include "stage3r.cuh"
#include "fullmetric.cuh"

namespace twoldg {

constexpr int kStageThreads = 256;
constexpr int kMaxGrid = 152 * 64;

template <typename T>
inline const ElementTables<T>& pick(const ElementTables<double>& a, const ElementTables<float>& b);
template <>
inline const ElementTables<double>& pick<double>(const ElementTables<double>& a, const ElementTables<float>&) {
    return a;
}
template <>
inline const ElementTables<float>& pick<float>(const ElementTables<double>&, const ElementTables<float>& b) {
    return b;
}

inline int grid_for(int64_t work, int threads) {
    int64_t g = (work + threads - 1) / threads;
    return (int)std::max<int64_t>(1, std::min<int64_t>(g, kMaxGrid));
}

template <typename T, int D, int P, bool COMP>
class OpsImpl : public Ops {
    Tab<T, P> tb_;
    CfTab<T, P> ct_;
    ElementTables<T> et_;

public:
    int max_smem_ = 0;

    explicit OpsImpl(const ElementTables<T>& t) : et_(t) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&max_smem_, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        cudaFuncSetAttribute(stage_kernel<T, D, P, COMP>, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem_);
        cudaFuncSetAttribute(stage_kernel_c<T, D, P, 2, COMP>, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem_);
        cudaFuncSetAttribute(stage_kernel_c<T, D, P, 4, COMP>, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem_);
        if constexpr (D == 3) {
            set_attrs(stage3r_kernel<T, P, 2, COMP>);
            set_attrs(stage3r_kernel<T, P, 4, COMP>);
            set_attrs(fm_gradient_kernel<T, P>);
            set_attrs(fm_stage_kernel<T, P, COMP>);
            set_attrs(fm_truncate_kernel<T, P>);
            // Legendre L_q, q < P, at the Gauss-Lobatto nodes, for the full metric's truncation
            for (int i = 0; i <= P; ++i) {
                double x = (double)t.nodes[i], l0 = 1, l1 = x;
                for (int q = 0; q < P; ++q) {
                    double lq = q == 0 ? l0 : q == 1 ? l1 : 0;
                    if (q >= 2) {
                        double a = 1, b = x;
                        for (int kk = 2; kk <= q; ++kk) { double c = ((2 * kk - 1) * x * b - (kk - 1) * a) / kk; a = b; b = c; }
                        lq = b;
                    }
                    ft_.L[q][i] = (T)lq;
                }
            }
        }
        // the stage kernels hold whole blocks in shared memory: take the largest carveout
        cudaFuncSetAttribute(stage_kernel<T, D, P, COMP>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
        cudaFuncSetAttribute(stage_kernel_c<T, D, P, 2, COMP>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
        cudaFuncSetAttribute(stage_kernel_c<T, D, P, 4, COMP>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
        cudaFuncSetAttribute(energy_kernel<T, D, P>, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem_);
        cudaFuncSetAttribute(truncate_kernel<T, D, P>, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem_);
        cudaGetLastError();
        const int P1 = P + 1, PW = P + 3;
        for (int i = 0; i < P1; ++i) {
            for (int k = 0; k < PW; ++k) tb_.W[i][k] = t.stencil[i * PW + k];
            tb_.tm[i] = t.topmode[i];
            tb_.td[i] = t.topdual[i];
            tb_.wq[i] = t.weights[i];
        }
        for (int r = 0; r < 2 * P1; ++r)
            for (int j = 0; j < P1; ++j) {
                ct_.I[r][j] = t.prolong[r * P1 + j];
                ct_.R[j][r] = t.restrict_[j * 2 * P1 + r];
            }
    }

    // padded u / gradient arrays: x pitch N+3, other dims N+2; ghost-free v: x pitch N+1
    static size_t padded_words(int E) {
        size_t N = (size_t)E * (P + 1), SS = N + 3;
        for (int k = 1; k < D; ++k) SS *= N + 2;
        return SS;
    }
    static size_t plain_words(int E) {
        size_t N = (size_t)E * (P + 1), LS = N + 1;
        for (int k = 1; k < D; ++k) LS *= N;
        return LS;
    }
    static size_t smem_words(int E) { return 2 * padded_words(E) + plain_words(E); }
    template <typename K>
    void set_attrs(K kern) {
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem_);
        cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    }
    int threads_ = 0;  // 0: the default for the shape
    void set_threads(int t) override { threads_ = t; }
    int default_threads(int E) const {
        size_t N = (size_t)E * (P + 1), NN = 1;
        for (int k = 0; k < D; ++k) NN *= N;
        if (NN >= 2048) return sizeof(T) == 8 ? 512 : 256;
        if (NN >= 256) return 128;
        return 64;
    }
    size_t stage_smem(int E) const override { return smem_words(E) * sizeof(T); }
    int stage_threads() const override { return threads_ ? threads_ : kStageThreads; }

    cudaError_t export_faces(const BlockItem* items, int nitems, int E, const void* u, void* fu, void* fog,
                             cudaStream_t s) const override {
        int64_t F = 1;
        for (int k = 0; k < D - 1; ++k) F *= (int64_t)E * (P + 1);
        int64_t work = (int64_t)nitems * 2 * D * F;
        export_faces_kernel<T, D, P><<<grid_for(work, 256), 256, 0, s>>>(
            items, nitems, E, (const T*)u, (T*)fu, (T*)fog, tb_);
        return cudaGetLastError();
    }

    cudaError_t cf_ghosts(const CfFace* cf, int ncf, int E, const void* fu, const void* fog, void* ugd, void* gfd,
                          void* ggd, cudaStream_t s) const override {
        if (ncf == 0) return cudaSuccess;
        int64_t F = 1;
        for (int k = 0; k < D - 1; ++k) F *= (int64_t)E * (P + 1);
        int g = grid_for((int64_t)ncf * F, 256);
        cf_ghost_u_kernel<T, D, P><<<g, 256, 0, s>>>(cf, ncf, E, (const T*)fu, (const T*)fog, (T*)ugd, (T*)gfd,
                                                    tb_, ct_);
        cf_ghost_g_kernel<T, D, P><<<g, 256, 0, s>>>(cf, ncf, E, (const T*)gfd, (T*)ggd, ct_);
        return cudaGetLastError();
    }

    cudaError_t stage(const BlockItem* items, int nitems, int E, int mode, int truncate, const StagePtrs& p,
                      int grid, cudaStream_t s) const override {
        StageArgs<T> a;
        a.items = items;
        a.nitems = nitems;
        a.E = E;
        a.mode = mode;
        a.truncate = truncate;
        a.u = (T*)p.u;
        a.y = (T*)p.y;
        a.acc = (T*)p.acc;
        a.comp = (T*)p.comp;
        a.du = (T*)p.du;
        a.fu_in = (const T*)p.fu_in;
        a.fog_in = (const T*)p.fog_in;
        a.fu_out = (T*)p.fu_out;
        a.fog_out = (T*)p.fog_out;
        a.ugd = (const T*)p.ugd;
        a.ggd = (const T*)p.ggd;
        a.rk = (const T*)p.rk;
        a.partial = p.partial;
        a.coef = (const T*)p.coef;
        a.trm = (const T*)p.trm;
        a.trd = (const T*)p.trd;
        size_t smem = stage_smem(E);
        if (smem > (size_t)max_smem_) return cudaErrorInvalidConfiguration;
        if (grid <= 0) grid = std::min(nitems, kMaxGrid);
        // the vector path needs 16-byte aligned state pointers
        uintptr_t al = (uintptr_t)p.u | (uintptr_t)p.y | (uintptr_t)p.acc | (uintptr_t)p.comp | (uintptr_t)p.du;
        const bool aligned = (al & 15) == 0;
        int nt = threads_ ? threads_ : default_threads(E);
        // the whole-lines-in-registers 3D kernel serves flat problems
        if constexpr (D == 3) {
            if (!p.coef && aligned && E == 2 && Stage3R<T, P, 2, COMP>::usable) {
                using S = Stage3R<T, P, 2, COMP>;
                stage3r_kernel<T, P, 2, COMP><<<grid, S::NT, S::words * sizeof(T), s>>>(a, tb_);
                return cudaGetLastError();
            }
            if (!p.coef && aligned && E == 4 && Stage3R<T, P, 4, COMP>::usable) {
                using S = Stage3R<T, P, 4, COMP>;
                stage3r_kernel<T, P, 4, COMP><<<grid, S::NT, S::words * sizeof(T), s>>>(a, tb_);
                return cudaGetLastError();
            }
        }
        if (aligned && E == 2) {
            stage_kernel_c<T, D, P, 2, COMP><<<grid, StageLaunch<T, D, P, 2>::NT, smem, s>>>(a, tb_);
        } else if (aligned && E == 4) {
            stage_kernel_c<T, D, P, 4, COMP><<<grid, StageLaunch<T, D, P, 4>::NT, smem, s>>>(a, tb_);
        } else {
            stage_kernel<T, D, P, COMP><<<grid, std::min(nt, 256), smem, s>>>(a, tb_);
        }
        return cudaGetLastError();
    }

    cudaError_t energy(const BlockItem* items, int nitems, int E, const StagePtrs& p,
                       cudaStream_t s) const override {
        StageArgs<T> a{};
        a.items = items;
        a.nitems = nitems;
        a.E = E;
        a.u = (T*)p.u;
        a.fu_in = (const T*)p.fu_in;
        a.fog_in = (const T*)p.fog_in;
        a.ugd = (const T*)p.ugd;
        a.ggd = (const T*)p.ggd;
        a.partial = p.partial;
        a.coef = (const T*)p.coef;
        size_t smem = (padded_words(E) + 1) * sizeof(T) + 32 * sizeof(double) + 16;
        auto kern = energy_kernel<T, D, P>;
        if (smem > (size_t)max_smem_) return cudaErrorInvalidConfiguration;
        kern<<<std::min(nitems, kMaxGrid), 256, smem, s>>>(a, tb_);
        return cudaGetLastError();
    }

    cudaError_t norm(const BlockItem* items, int nitems, int E, const void* u, const void* ref, int p,
                     int vars_mask, double* num, double* vol, const void* coef, int ncoef,
                     cudaStream_t s) const override {
        norm_kernel<T, D, P><<<std::min(nitems, kMaxGrid), 256, 0, s>>>(
            items, nitems, E, (const T*)u, (const T*)ref, p, vars_mask, tb_, num, vol, (const T*)coef, ncoef);
        return cudaGetLastError();
    }

    cudaError_t truncate(const BlockItem* items, int nitems, int E, void* u, const void* trm, const void* trd,
                         cudaStream_t s) const override {
        size_t smem = plain_words(E) * sizeof(T);
        auto kern = truncate_kernel<T, D, P>;
        if (smem > (size_t)max_smem_) return cudaErrorInvalidConfiguration;
        kern<<<std::min(nitems, kMaxGrid), 256, smem, s>>>(items, nitems, E, (T*)u, tb_, (const T*)trm,
                                                          (const T*)trd);
        return cudaGetLastError();
    }

    // ---- full metric (3D)
    FmTab<T, P> ft_;
    FmArgs<T> fm_args(const BlockItem* items, int nitems, int E, int mode, int truncate, const FmPtrs& p) const {
        FmArgs<T> a{};
        a.items = items;
        a.nitems = nitems;
        a.E = E;
        a.mode = mode;
        a.truncate = truncate;
        a.u = (T*)p.u;
        a.y = (T*)p.y;
        a.acc = (T*)p.acc;
        a.comp = (T*)p.comp;
        a.du = (T*)p.du;
        a.fu_in = (const T*)p.fu_in;
        a.fu_out = (T*)p.fu_out;
        a.V = (T*)p.V;
        a.fv = (T*)p.fv;
        a.coef = (const T*)p.coef;
        a.rk = (const T*)p.rk;
        a.tinfo = p.tinfo;
        a.bnd_x = p.bnd_x;
        for (int q = 0; q < 3; ++q) a.wave.k[q] = p.wave_k[q];
        a.wave.omega = std::sqrt(p.wave_k[0] * p.wave_k[0] + p.wave_k[1] * p.wave_k[1] + p.wave_k[2] * p.wave_k[2]);
        a.wave.phi = p.wave_phi;
        a.eslot = p.eslot;
        a.ew = (const T*)p.ew;
        a.echol = (const T*)p.echol;
        a.partial = p.partial;
        return a;
    }
    static size_t fm_grad_smem(int E) { return (padded_words(E) + 3 * plain_words(E)) * sizeof(T); }
    static size_t fm_stage_smem(int E) {
        size_t m3 = (size_t)P * P * P, EE = (size_t)E * E * E;
        return (padded_words(E) + 2 * plain_words(E) + EE * m3) * sizeof(T);
    }
    cudaError_t fm_gradient(const BlockItem* items, int nitems, int E, int mode, const FmPtrs& p,
                            cudaStream_t s) const override {
        if constexpr (D != 3) return cudaErrorNotSupported;
        else {
            size_t smem = fm_grad_smem(E);
            if (smem > (size_t)max_smem_) return cudaErrorInvalidConfiguration;
            fm_gradient_kernel<T, P><<<std::min(nitems, kMaxGrid), 256, smem, s>>>(
                fm_args(items, nitems, E, mode, 0, p), tb_);
            return cudaGetLastError();
        }
    }
    cudaError_t fm_stage(const BlockItem* items, int nitems, int E, int mode, int truncate, const FmPtrs& p,
                         cudaStream_t s) const override {
        if constexpr (D != 3) return cudaErrorNotSupported;
        else {
            size_t smem = fm_stage_smem(E);
            if (smem > (size_t)max_smem_) return cudaErrorInvalidConfiguration;
            fm_stage_kernel<T, P, COMP><<<std::min(nitems, kMaxGrid), 256, smem, s>>>(
                fm_args(items, nitems, E, mode, truncate, p), tb_, ft_);
            return cudaGetLastError();
        }
    }
    cudaError_t fm_truncate(const BlockItem* items, int nitems, int E, const FmPtrs& p,
                            cudaStream_t s) const override {
        if constexpr (D != 3) return cudaErrorNotSupported;
        else {
            size_t smem = (plain_words(E) + (size_t)E * E * E * P * P * P) * sizeof(T);
            if (smem > (size_t)max_smem_) return cudaErrorInvalidConfiguration;
            fm_truncate_kernel<T, P><<<std::min(nitems, kMaxGrid), 256, smem, s>>>(
                fm_args(items, nitems, E, 0, 1, p), tb_, ft_);
            return cudaGetLastError();
        }
    }
    cudaError_t fm_energy(const BlockItem* items, int nitems, int E, const FmPtrs& p, cudaStream_t s) const override {
        if constexpr (D != 3) return cudaErrorNotSupported;
        else {
            fm_energy_kernel<T, P><<<std::min(nitems, kMaxGrid), 256, 0, s>>>(fm_args(items, nitems, E, 5, 0, p),
                                                                              tb_);
            return cudaGetLastError();
        }
    }

    cudaError_t maxabs(const BlockItem* items, int nitems, int E, const void* u, int var, double* part,
                       cudaStream_t s) const override {
        int NN = 1;
        for (int k = 0; k < D; ++k) NN *= E * (P + 1);
        maxabs_kernel<T, D><<<std::min(nitems, kMaxGrid), 256, 0, s>>>(items, nitems, NN, (const T*)u, var, part);
        return cudaGetLastError();
    }

    cudaError_t modes(const BlockItem* items, int nitems, int E, const void* u, int var, int nq, const int* modes,
                      const double* weights, const double* pows, double post, void* tau,
                      cudaStream_t s) const override {
        if (nq < 1 || nq > P + 1) return cudaErrorInvalidValue;
        ModeTab<T, P> mt{};
        for (int q = 0; q < nq; ++q) {
            for (int j = 0; j <= P; ++j) mt.dual[q][j] = et_.duals[modes[q] * (P + 1) + j];
            mt.weight[q] = (T)weights[q];
            mt.pw[q] = (T)pows[q];
        }
        mt.nq = nq;
        mt.post = (T)post;
        int64_t EE = 1;
        for (int k = 0; k < D; ++k) EE *= E;
        mode_kernel<T, D, P><<<grid_for((int64_t)nitems * EE, 128), 128, 0, s>>>(items, nitems, E, (const T*)u,
                                                                                 var, mt, (T*)tau);
        return cudaGetLastError();
    }
};

template <int D, int P>
Ops* make_ops_p(int prec, const ElementTables<double>& t64, const ElementTables<float>& t32) {
    switch (prec) {
        case PREC_F64: return new OpsImpl<double, D, P, false>(t64);
        case PREC_F32: return new OpsImpl<float, D, P, false>(t32);
        case PREC_F32C: return new OpsImpl<float, D, P, true>(t32);
        default: return nullptr;
    }
}

template <int D>
Ops* make_ops_dim(int prec, int P, const ElementTables<double>& t64, const ElementTables<float>& t32) {
    switch (P) {
        case 1: return make_ops_p<D, 1>(prec, t64, t32);
        case 2: return make_ops_p<D, 2>(prec, t64, t32);
        case 3: return make_ops_p<D, 3>(prec, t64, t32);
        case 4: return make_ops_p<D, 4>(prec, t64, t32);
        case 5: return make_ops_p<D, 5>(prec, t64, t32);
        case 6: return make_ops_p<D, 6>(prec, t64, t32);
        default: return nullptr;
    }
}

}  // namespace twoldg
