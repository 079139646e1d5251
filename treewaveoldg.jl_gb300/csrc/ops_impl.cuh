// The templated Ops implementation: fills the constant tables once and
// launches the kernels of kernels.cuh with them.
#pragma once
#include <algorithm>
#include <cmath>

#include "kernels.cuh"
#include "ops.h"
#include "stage3r.cuh"
#include "stage2r.cuh"
#include "fullmetric.cuh"

namespace twoldg {

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
    // the register-line and fixed-shape stage kernels are built for P <= 6;
    // higher orders run the run-time-shape kernel
    static constexpr bool kShaped = P <= 6;
    Tab<T, P> tb_;
    CfTab<T, P> ct_;
    ElementTables<T> et_;

public:
    int max_smem_ = 0;

    explicit OpsImpl(const ElementTables<T>& t) : et_(t) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&max_smem_, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        cudaDeviceGetAttribute(&nsm_, cudaDevAttrMultiProcessorCount, dev);
        set_attrs(stage_kernel<T, D, P, COMP>);
        if constexpr (kShaped) {
            set_attrs(stage_kernel_c<T, D, P, 2, COMP>);
            set_attrs(stage_kernel_c<T, D, P, 4, COMP>);
        }
        if constexpr (D == 2 && kShaped) {
            set_attrs2r<2>();
            set_attrs2r<4>();
        }
        if constexpr (D == 3 && kShaped) {
            set_attrs3r<2>();
            set_attrs3r<4>();
            if constexpr (sizeof(T) == 4) stage3r_cf_attrs<T, P, COMP>(max_smem_);
        }
        if constexpr (D == 3) {
            set_attrs(fm_gradient_kernel<T, P>);
            if constexpr (kShaped) {
                if constexpr (Stage3R<T, P, 2, false>::usable) set_attrs(fm_gradient_r_kernel<T, P, 2>);
                if constexpr (Stage3R<T, P, 4, false>::usable) set_attrs(fm_gradient_r_kernel<T, P, 4>);
                fm_stage_r_attrs<T, P, 2, COMP>(max_smem_);
                fm_stage_r_attrs<T, P, 4, COMP>(max_smem_);
            }
            set_attrs(fm_stage_kernel<T, P, COMP>);
            set_attrs(fm_stage_kernel<T, P, COMP, 1>);
            set_attrs(fm_stage_kernel<T, P, COMP, 2>);
            set_attrs(fm_stage_kernel<T, P, COMP, 3>);
            set_attrs(fm_stage_kernel<T, P, COMP, 4>);
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
        // the energy and truncation kernels stage blocks in shared memory too
        set_attrs(energy_kernel<T, D, P>);
        set_attrs(truncate_kernel<T, D, P>);
        set_attrs(mode_staged_kernel<T, D, P>);
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
    // the kernels hold whole blocks in shared memory: the largest carveout, and
    // as dynamic shared memory the opt-in maximum less the kernel's own static
    template <typename K>
    void set_attrs(K kern) {
        cudaFuncAttributes fa{};
        cudaFuncGetAttributes(&fa, kern);
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             max_smem_ - (int)fa.sharedSizeBytes);
        cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    }
    Launch launch_{0, 0, 0};
    int grid_cap_ = 0;  // 0: one CTA per block (at most kMaxGrid)
    int nsm_ = 0;
    int default_threads(int E) const {
        size_t N = (size_t)E * (P + 1), NN = 1;
        for (int k = 0; k < D; ++k) NN *= N;
        if (NN >= 2048) return sizeof(T) == 8 ? 512 : 256;
        if (NN >= 256) return 128;
        return 64;
    }
    size_t stage_smem(int E) const override { return smem_words(E) * sizeof(T); }

    // the kernel that runs for a requested one: the register-line kernel for
    // flat 3D blocks of E = 2 or 4 whose cross-section fits a CTA, the
    // fixed-shape kernel for E = 2 or 4, the run-time-shape kernel always;
    // 0 or a kernel the shape cannot take means the first that it can
    int resolve(int kernel, int E, bool flat, bool aligned) const {
        bool line = false;
        if constexpr (D == 3 && kShaped) {
            line = flat && aligned && ((E == 2 && Stage3R<T, P, 2, COMP>::usable) ||
                                       (E == 4 && Stage3R<T, P, 4, COMP>::usable));
        }
        if constexpr (D == 2 && kShaped) {
            line = flat && aligned && ((E == 2 && Stage2R<T, P, 2, COMP>::usable) ||
                                       (E == 4 && Stage2R<T, P, 4, COMP>::usable));
        }
        const bool fixed = kShaped && aligned && (E == 2 || E == 4);
        if (kernel == 1 && line) return 1;
        if (kernel == 2 && fixed) return 2;
        if (kernel == 3) return 3;
        return line ? 1 : fixed ? 2 : 3;
    }
    int run_threads(int kernel, int E) const {
        if (kernel == 1 && D == 2) return E == 2 ? Stage2R<T, P, 2, false>::NT : Stage2R<T, P, 4, false>::NT;
        if (kernel == 1) return E * (P + 1) * E * (P + 1);
        if (kernel == 2) return E == 2 ? StageLaunch<T, D, P, 2>::NT : StageLaunch<T, D, P, 4>::NT;
        return std::min(launch_.threads ? launch_.threads : default_threads(E), 256);
    }
    // CTAs of the resolved kernel one SM holds at once
    int resident(int kernel, int threads, int E) const {
        int n = 0;
        if constexpr (D == 3 && kShaped) {
            if (kernel == 1) {
                // the stages between the first and the last
                if (E == 2)
                    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, stage3r_kernel<T, P, 2, false, false, 2>,
                                                                  threads, Stage3R<T, P, 2, false>::words * sizeof(T));
                else
                    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, stage3r_kernel<T, P, 4, false, false, 2>,
                                                                  threads, Stage3R<T, P, 4, false>::words * sizeof(T));
                return n;
            }
        }
        if constexpr (D == 2 && kShaped) {
            if (kernel == 1) {
                if (E == 2)
                    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, stage2r_kernel<T, P, 2, false, 2>, threads,
                                                                  Stage2R<T, P, 2, false>::words * sizeof(T));
                else
                    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, stage2r_kernel<T, P, 4, false, 2>, threads,
                                                                  Stage2R<T, P, 4, false>::words * sizeof(T));
                return n;
            }
        }
        if constexpr (kShaped) {
            if (kernel == 2) {
                if (E == 2)
                    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, stage_kernel_c<T, D, P, 2, COMP>, threads,
                                                                  stage_smem(E));
                else
                    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, stage_kernel_c<T, D, P, 4, COMP>, threads,
                                                                  stage_smem(E));
                return n;
            }
        }
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, stage_kernel<T, D, P, COMP>, threads, stage_smem(E));
        return n;
    }
    void set_launch(const Launch& l, int E, bool flat) override {
        launch_ = l;
        grid_cap_ = 0;
        if (l.waves > 0) {
            const int k = resolve(l.kernel, E, flat, true);
            const int r = resident(k, run_threads(k, E), E);
            cudaGetLastError();
            grid_cap_ = std::max(1, l.waves * std::max(r, 1) * std::max(nsm_, 1));
        }
    }
    Launch launch() const override { return launch_; }
    int launch_candidates(int E, bool flat, Launch* out, int max) const override {
        int n = 0;
        auto add = [&](int k, int t, int w) {
            if (n < max) out[n++] = Launch{k, t, w};
        };
        for (int k = 1; k <= 3; ++k) {
            if (resolve(k, E, flat, true) != k) continue;
            if (k < 3) {
                for (int w = 0; w <= 2; ++w) add(k, 0, w);
            } else {
                for (int t : {64, 128, 256})
                    for (int w = 0; w <= 1; ++w) add(k, t, w);
            }
        }
        return n;
    }

    cudaError_t export_faces(const BlockItem* items, int nitems, int E, const void* u, void* fu, void* fog,
                             cudaStream_t s) const override {
        int64_t F = 1;
        for (int k = 0; k < D - 1; ++k) F *= (int64_t)E * (P + 1);
        int64_t work = (int64_t)nitems * 2 * D * F;
        export_faces_kernel<T, D, P><<<grid_for(work, 256), 256, 0, s>>>(
            items, nitems, E, (const T*)u, (T*)fu, (T*)fog, tb_);
        return cudaGetLastError();
    }

    cudaError_t gather(const void* u, int64_t varoff, int64_t npoints, int nper, const int64_t* index,
                       const void* w, void* out, cudaStream_t s) const override {
        if (npoints == 0) return cudaSuccess;
        gather_kernel<T><<<grid_for(npoints, 256), 256, 0, s>>>((const T*)u, varoff, npoints, nper, index,
                                                                 (const T*)w, (T*)out);
        return cudaGetLastError();
    }

    cudaError_t transfer(const TransferItem* items, int nitems, int E, const void* src, void* dst,
                         cudaStream_t s) const override {
        if (nitems == 0) return cudaSuccess;
        transfer_kernel<T, D, P><<<std::min(nitems, kMaxGrid), 256, 0, s>>>(items, nitems, E, (const T*)src,
                                                                          (T*)dst, ct_);
        return cudaGetLastError();
    }

    cudaError_t cf_ghosts(const CfFace* cf, int ncf, int E, const void* fu, const void* fog, void* ugd, void* gfd,
                          void* ggd, cudaStream_t s) const override {
        if (ncf == 0) return cudaSuccess;
        int64_t F = 1;
        for (int k = 0; k < D - 1; ++k) F *= (int64_t)E * (P + 1);
        (void)gfd;  // the composite images need no intermediate plane
        const size_t smem = (size_t)(1 << (D - 1)) * F * sizeof(T);
        cf_ghost_kernel<T, D, P><<<std::min(ncf, kMaxGrid), 128, smem, s>>>(cf, ncf, E, (const T*)fu, (const T*)fog,
                                                                           (T*)ugd, (T*)ggd, tb_, ct_);
        return cudaGetLastError();
    }

    cudaError_t cf_planes(const CfFace* cf, int ncf, int E, const void* src, void* dst, int vars,
                          cudaStream_t s) const override {
        if (ncf == 0) return cudaSuccess;
        int64_t F = 1;
        for (int k = 0; k < D - 1; ++k) F *= (int64_t)E * (P + 1);
        int g = grid_for((int64_t)ncf * vars * F, 256);
        cf_plane_kernel<T, D, P><<<g, 256, 0, s>>>(cf, ncf, E, vars, (const T*)src, (T*)dst, ct_);
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
        a.cf = nullptr;
        a.cfidx = nullptr;
        a.gsd = (const T*)p.gsd;
        a.ugd_out = (T*)p.ugd_out;
        a.ggd_out = (T*)p.ggd_out;
        a.gsd_out = (T*)p.gsd_out;
        size_t smem = stage_smem(E);
        if (smem > (size_t)max_smem_) return cudaErrorInvalidConfiguration;
        if (grid <= 0) grid = std::min(nitems, grid_cap_ > 0 ? grid_cap_ : kMaxGrid);
        // the fixed-shape kernels need 16-byte aligned state pointers
        uintptr_t al = (uintptr_t)p.u | (uintptr_t)p.y | (uintptr_t)p.acc | (uintptr_t)p.comp | (uintptr_t)p.du;
        const bool aligned = (al & 15) == 0;
        const int k = resolve(launch_.kernel, E, !p.coef, aligned);
        if (p.cf && p.ncf > 0) {
            // the 3D register-line kernel's FP32 RK stages read the planes the
            // previous stage's epilogues wrote and write the next stage's;
            // the others (FP64 among them: bound by the FP64 pipe, they
            // measured faster so) read complete planes a launch of their own
            // fills
            if constexpr (D == 3 && kShaped && sizeof(T) == 4) {
                if (k == 1 && (E == 2 || E == 4) && mode != MODE_RHS && p.ugd_out) {
                    a.cf = p.cf;
                    a.cfidx = p.cfidx;
                    if (E == 2) return stage3r_cf_launch<T, P, 2, COMP>(a, tb_, ct_, grid, mode, s, p.pdl);
                    return stage3r_cf_launch<T, P, 4, COMP>(a, tb_, ct_, grid, mode, s, p.pdl);
                }
            }
            cudaError_t e = cf_ghosts(p.cf, p.ncf, E, p.fu_in, p.fog_in, const_cast<void*>(p.ugd), nullptr,
                                      const_cast<void*>(p.ggd), s);
            if (e != cudaSuccess) return e;
        }
        if constexpr (D == 3 && kShaped) {
            if (k == 1 && E == 2) return launch3r<2>(a, grid, mode, s, p.pdl);
            if (k == 1 && E == 4) return launch3r<4>(a, grid, mode, s, p.pdl);
        }
        if constexpr (D == 2 && kShaped) {
            if (k == 1 && E == 2) return launch2r<2>(a, grid, mode, s, p.pdl);
            if (k == 1 && E == 4) return launch2r<4>(a, grid, mode, s, p.pdl);
        }
        if constexpr (kShaped) {
            if (k == 2 && E == 2) {
                stage_kernel_c<T, D, P, 2, COMP><<<grid, StageLaunch<T, D, P, 2>::NT, smem, s>>>(a, tb_);
                return cudaGetLastError();
            }
            if (k == 2 && E == 4) {
                stage_kernel_c<T, D, P, 4, COMP><<<grid, StageLaunch<T, D, P, 4>::NT, smem, s>>>(a, tb_);
                return cudaGetLastError();
            }
        }
        stage_kernel<T, D, P, COMP><<<grid, run_threads(3, E), smem, s>>>(a, tb_);
        return cudaGetLastError();
    }

    // The register-line kernel: stage 4 of the compensated path with the
    // compensation array, stage 1 in the lean variant where that fits one more
    // CTA per SM, every other stage without the compensation array.
    // One instantiation per stage (its data flow compiled in, no other's).
    template <int E>
    cudaError_t launch3r(const StageArgs<T>& a, int grid, int mode, cudaStream_t s, bool pdl) const {
        if constexpr (D == 3) {
            using SL = Stage3R<T, P, E, false, true>;
            using S0 = Stage3R<T, P, E, false>;
            using SC = Stage3R<T, P, E, true>;
            const size_t m0 = S0::words * sizeof(T);
            auto go = [&](auto kern, int nt, size_t sm) {
                StageArgs<T> b = a;
                b.release = pdl && release_early(kern, grid, nt, sm);
                return launch_kernel(kern, grid, nt, sm, s, pdl, b, tb_, ct_);
            };
            if constexpr (COMP) {
                if (mode == MODE_STAGE4) {
                    go(stage3r_kernel<T, P, E, true, false, 4>, SC::NT, SC::words * sizeof(T));
                    return cudaGetLastError();
                }
            }
            if (mode == MODE_STAGE1) {
                if constexpr (SL::MINB > S0::MINB)
                    go(stage3r_kernel<T, P, E, false, true, 1>, SL::NT, SL::words * sizeof(T));
                else
                    go(stage3r_kernel<T, P, E, false, false, 1>, S0::NT, m0);
            } else if (mode == 2) {
                if constexpr (SL::MINB > S0::MINB)
                    go(stage3r_kernel<T, P, E, false, true, 2>, SL::NT, SL::words * sizeof(T));
                else
                    go(stage3r_kernel<T, P, E, false, false, 2>, S0::NT, m0);
            } else if (mode == 3) {
                go(stage3r_kernel<T, P, E, false, false, 3>, S0::NT, m0);
            } else if (mode == MODE_STAGE4) {
                go(stage3r_kernel<T, P, E, false, false, 4>, S0::NT, m0);
            } else {
                go(stage3r_kernel<T, P, E, false>, S0::NT, m0);
            }
        }
        return cudaGetLastError();
    }
    // The 2D register-line kernel: K blocks a CTA, so the grid is the items
    // over K (capped by the persistent layout's CTAs); stage 4 of the
    // compensated path with the compensation array.
    template <int E>
    cudaError_t launch2r(const StageArgs<T>& a, int grid, int mode, cudaStream_t s, bool pdl) const {
        if constexpr (D == 2) {
            using S0 = Stage2R<T, P, E, false>;
            using SC = Stage2R<T, P, E, true>;
            const int g = std::max(1, std::min(grid, (a.nitems + S0::K - 1) / S0::K));
            const size_t m0 = S0::words * sizeof(T);
            auto go = [&](auto kern, int nt, size_t sm) {
                StageArgs<T> b = a;
                b.release = pdl && release_early(kern, g, nt, sm);
                return launch_kernel(kern, g, nt, sm, s, pdl, b, tb_);
            };
            if constexpr (COMP) {
                if (mode == MODE_STAGE4) {
                    go(stage2r_kernel<T, P, E, true, 4>, SC::NT, SC::words * sizeof(T));
                    return cudaGetLastError();
                }
            }
            if (mode == MODE_STAGE1)
                go(stage2r_kernel<T, P, E, false, 1>, S0::NT, m0);
            else if (mode == 2)
                go(stage2r_kernel<T, P, E, false, 2>, S0::NT, m0);
            else if (mode == 3)
                go(stage2r_kernel<T, P, E, false, 3>, S0::NT, m0);
            else if (mode == MODE_STAGE4)
                go(stage2r_kernel<T, P, E, false, 4>, S0::NT, m0);
            else
                go(stage2r_kernel<T, P, E, false>, S0::NT, m0);
        }
        return cudaGetLastError();
    }
    template <int E>
    void set_attrs2r() {
        if constexpr (D == 2) {
            if constexpr (COMP) set_attrs(stage2r_kernel<T, P, E, true, 4>);
            set_attrs(stage2r_kernel<T, P, E, false>);
            set_attrs(stage2r_kernel<T, P, E, false, 1>);
            set_attrs(stage2r_kernel<T, P, E, false, 2>);
            set_attrs(stage2r_kernel<T, P, E, false, 3>);
            if constexpr (!COMP) set_attrs(stage2r_kernel<T, P, E, false, 4>);
        }
    }
    template <int E>
    void set_attrs3r() {
        if constexpr (D == 3) {
            if constexpr (COMP) set_attrs(stage3r_kernel<T, P, E, true, false, 4>);
            set_attrs(stage3r_kernel<T, P, E, false>);
            set_attrs(stage3r_kernel<T, P, E, false, false, 2>);
            if constexpr (Stage3R<T, P, E, false, true>::MINB > Stage3R<T, P, E, false>::MINB)
                set_attrs(stage3r_kernel<T, P, E, false, true, 2>);
            set_attrs(stage3r_kernel<T, P, E, false, false, 3>);
            if constexpr (!COMP) set_attrs(stage3r_kernel<T, P, E, false, false, 4>);
            if constexpr (Stage3R<T, P, E, false, true>::MINB > Stage3R<T, P, E, false>::MINB)
                set_attrs(stage3r_kernel<T, P, E, false, true, 1>);
            else
                set_attrs(stage3r_kernel<T, P, E, false, false, 1>);
        }
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
        a.M = (const T*)p.M;
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
        a.boundary = p.boundary;
        a.kappa = (T)p.kappa;
        a.inv_r = (T)p.inv_r;
        a.fslot = p.fslot;
        a.fradial = p.fradial;
        a.frm = (const T*)p.frm;
        a.frd = (const T*)p.frd;
        a.faslot = p.faslot;
        a.faw = (const T*)p.faw;
        a.fachol = (const T*)p.fachol;
        a.bidx = p.bidx;
        a.btab = p.btab;
        a.ugd = (const T*)p.ugd;
        a.vgd = (const T*)p.vgd;
        return a;
    }
    static size_t fm_grad_smem(int E) { return (padded_words(E) + 3 * plain_words(E)) * sizeof(T); }
    // coefficients per element: P^3 (per-element projection) or (P+1) P^2 (factored)
    static size_t fm_cbuf_words(int E) { return (size_t)E * E * E * (P + 1) * P * P; }
    static size_t fm_stage_smem(int E) { return (padded_words(E) + 2 * plain_words(E) + fm_cbuf_words(E)) * sizeof(T); }
    // Whether the register-line full-metric passes on 8^3 blocks (64 threads a
    // CTA) have threads enough to fill the GPU: in FP32 a forest whose blocks
    // give every SM fewer than 1024 threads (half what it holds) runs the
    // run-time-shape passes of 256 threads a CTA instead (the seven-patch
    // ball, 448 blocks: 0.245 against 0.269 ms a step), while FP64, held by
    // its pipe, keeps the register-line passes at any size (0.463 against
    // 0.616 ms there).
    bool fm_r_fills(int nitems) const {
        return sizeof(T) == 8 || (int64_t)nitems * 64 >= (int64_t)nsm_ * 1024;
    }
    cudaError_t fm_gradient(const BlockItem* items, int nitems, int E, int mode, const FmPtrs& p,
                            cudaStream_t s) const override {
        if constexpr (D != 3) return cudaErrorNotSupported;
        else {
            const int g = std::min(nitems, kMaxGrid);
            if constexpr (kShaped) {
                // the register-line pass for the compile-time shapes
                auto go = [&](auto kern, int nt, size_t sm) {
                    FmArgs<T> b = fm_args(items, nitems, E, mode, 0, p);
                    b.release = p.pdl && release_early(kern, g, nt, sm);
                    launch_kernel(kern, g, nt, sm, s, p.pdl != 0, b, tb_);
                    return cudaGetLastError();
                };
                if (E == 2 && Stage3R<T, P, 2, false>::usable && fm_r_fills(nitems))
                    return go(fm_gradient_r_kernel<T, P, 2>, Stage3R<T, P, 2, false>::NT,
                              FmGradR<T, P, 2>::words * sizeof(T));
                if (E == 4 && Stage3R<T, P, 4, false>::usable &&
                    FmGradR<T, P, 4>::words * sizeof(T) <= (size_t)max_smem_)
                    return go(fm_gradient_r_kernel<T, P, 4>, Stage3R<T, P, 4, false>::NT,
                              FmGradR<T, P, 4>::words * sizeof(T));
            }
            size_t smem = fm_grad_smem(E);
            if (smem > (size_t)max_smem_) return cudaErrorInvalidConfiguration;
            fm_gradient_kernel<T, P><<<g, 256, smem, s>>>(fm_args(items, nitems, E, mode, 0, p), tb_);
            return cudaGetLastError();
        }
    }
    cudaError_t fm_stage(const BlockItem* items, int nitems, int E, int mode, int truncate, const FmPtrs& p,
                         cudaStream_t s) const override {
        if constexpr (D != 3) return cudaErrorNotSupported;
        else {
            size_t smem = fm_stage_smem(E);
            if (smem > (size_t)max_smem_) return cudaErrorInvalidConfiguration;
            const int g = std::min(nitems, kMaxGrid);
            const FmArgs<T> fa = fm_args(items, nitems, E, mode, truncate, p);
            if constexpr (kShaped) {
                // the register-line pass for the compile-time shapes' RK stages
                if (mode >= MODE_STAGE1 && mode <= MODE_STAGE4) {
                    if (E == 2 && Stage3R<T, P, 2, false>::usable && fm_r_fills(nitems) &&
                        fm_stage_r_smem<T, P, 2, COMP>() <= (size_t)max_smem_)
                        return fm_stage_r_launch<T, P, 2, COMP>(fa, tb_, ft_, g, mode, s, p.pdl != 0);
                    if (E == 4 && Stage3R<T, P, 4, false>::usable &&
                        fm_stage_r_smem<T, P, 4, COMP>() <= (size_t)max_smem_)
                        return fm_stage_r_launch<T, P, 4, COMP>(fa, tb_, ft_, g, mode, s, p.pdl != 0);
                }
            }
            // one instantiation per stage
            if (mode == MODE_STAGE1) fm_stage_kernel<T, P, COMP, 1><<<g, 256, smem, s>>>(fa, tb_, ft_);
            else if (mode == 2) fm_stage_kernel<T, P, COMP, 2><<<g, 256, smem, s>>>(fa, tb_, ft_);
            else if (mode == 3) fm_stage_kernel<T, P, COMP, 3><<<g, 256, smem, s>>>(fa, tb_, ft_);
            else if (mode == MODE_STAGE4) fm_stage_kernel<T, P, COMP, 4><<<g, 256, smem, s>>>(fa, tb_, ft_);
            else fm_stage_kernel<T, P, COMP><<<g, 256, smem, s>>>(fa, tb_, ft_);
            return cudaGetLastError();
        }
    }
    cudaError_t fm_truncate(const BlockItem* items, int nitems, int E, const FmPtrs& p,
                            cudaStream_t s) const override {
        if constexpr (D != 3) return cudaErrorNotSupported;
        else {
            size_t smem = (plain_words(E) + fm_cbuf_words(E)) * sizeof(T);
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
        int64_t EE = 1, NN = 1;
        for (int k = 0; k < D; ++k) {
            EE *= E;
            NN *= (int64_t)E * (P + 1);
        }
        // the block staged in shared memory where it fits, else one thread
        // an element reading global memory
        const size_t smem = ((size_t)((NN + 3) & ~3) + (size_t)D * EE * nq) * sizeof(T);
        if (smem <= (size_t)max_smem_) {
            mode_staged_kernel<T, D, P><<<std::min(nitems, kMaxGrid), 256, smem, s>>>(items, nitems, E,
                                                                                      (const T*)u, var, mt, (T*)tau);
        } else {
            mode_kernel<T, D, P><<<grid_for((int64_t)nitems * EE, 128), 128, 0, s>>>(items, nitems, E, (const T*)u,
                                                                                     var, mt, (T*)tau);
        }
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
        case 7: return make_ops_p<D, 7>(prec, t64, t32);
        case 8: return make_ops_p<D, 8>(prec, t64, t32);
        default: return nullptr;
    }
}

}  // namespace twoldg
