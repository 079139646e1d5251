// The register-line stage of a forest with refinement: the launches of the
// CFP instantiations of stage3r_kernel (coarse-fine ghost planes read as the
// previous stage's epilogues wrote them, the next stage's written in the
// block's epilogue) and their attributes. Only the forests with refinement run
// them, so they live in translation units of their own
// (kernels_d3_p<P>_cf.cu), which the build compiles beside the uniform ones,
// and the uniform kernels keep their code as it is.
#pragma once
#include "kernels.cuh"
#include "stage3r.cuh"

namespace twoldg {

template <typename K>
inline void stage3r_cf_attr(K kern, int max_smem) {
    cudaFuncAttributes fa{};
    cudaFuncGetAttributes(&fa, kern);
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem - (int)fa.sharedSizeBytes);
    cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
}

template <typename T, int P, int E, bool COMP>
inline void stage3r_cf_attrs_e(int max_smem) {
    if constexpr (Stage3R<T, P, E, false>::usable) {
        if constexpr (COMP) stage3r_cf_attr(stage3r_kernel<T, P, E, true, false, 4, true>, max_smem);
        stage3r_cf_attr(stage3r_kernel<T, P, E, false, false, 1, true>, max_smem);
        stage3r_cf_attr(stage3r_kernel<T, P, E, false, false, 2, true>, max_smem);
        stage3r_cf_attr(stage3r_kernel<T, P, E, false, false, 3, true>, max_smem);
        if constexpr (!COMP) stage3r_cf_attr(stage3r_kernel<T, P, E, false, false, 4, true>, max_smem);
    }
}

template <typename T, int P, bool COMP>
void stage3r_cf_attrs(int max_smem) {
    stage3r_cf_attrs_e<T, P, 2, COMP>(max_smem);
    stage3r_cf_attrs_e<T, P, 4, COMP>(max_smem);
}

// Every RK stage in the plain register budget (the lean stage 1 and 2
// variants of the uniform forests are left out here), as a programmatic
// dependent launch when `pdl` is set; the right-hand side of a forest with
// refinement runs the plain kernel after a launch that fills its ghost planes.
template <typename T, int P, int E, bool COMP>
cudaError_t stage3r_cf_launch(const StageArgs<T>& a, const Tab<T, P>& tb, const CfTab<T, P>& ct, int grid,
                              int mode, cudaStream_t s, bool pdl) {
    if constexpr (!Stage3R<T, P, E, false>::usable) {
        return cudaErrorInvalidConfiguration;
    } else {
        using S0 = Stage3R<T, P, E, false>;
        using SC = Stage3R<T, P, E, true>;
        const size_t m0 = S0::words * sizeof(T);
        auto go = [&](auto kern, int nt, size_t sm) {
            StageArgs<T> b = a;
            b.release = pdl && release_early(kern, grid, nt, sm);
            return launch_kernel(kern, grid, nt, sm, s, pdl, b, tb, ct);
        };
        if constexpr (COMP) {
            if (mode == MODE_STAGE4) {
                go(stage3r_kernel<T, P, E, true, false, 4, true>, SC::NT, SC::words * sizeof(T));
                return cudaGetLastError();
            }
        }
        if (mode == MODE_STAGE1)
            go(stage3r_kernel<T, P, E, false, false, 1, true>, S0::NT, m0);
        else if (mode == 2)
            go(stage3r_kernel<T, P, E, false, false, 2, true>, S0::NT, m0);
        else if (mode == 3)
            go(stage3r_kernel<T, P, E, false, false, 3, true>, S0::NT, m0);
        else if (mode == MODE_STAGE4)
            go(stage3r_kernel<T, P, E, false, false, 4, true>, S0::NT, m0);
        else
            return cudaErrorInvalidValue;
        return cudaGetLastError();
    }
}

// The instantiations of one order: FP32 and FP32 compensated (the FP64
// stages, bound by the FP64 pipe, fill their planes in a launch of their own,
// which measured faster there).
#define TWOLDG_STAGE3R_CF_E(T, P, E, COMP)                                                                      \
    template cudaError_t stage3r_cf_launch<T, P, E, COMP>(const StageArgs<T>&, const Tab<T, P>&,              \
                                                           const CfTab<T, P>&, int, int, cudaStream_t, bool);
#define TWOLDG_STAGE3R_CF(P)                                \
    template void stage3r_cf_attrs<float, P, false>(int);  \
    template void stage3r_cf_attrs<float, P, true>(int);   \
    TWOLDG_STAGE3R_CF_E(float, P, 2, false)                \
    TWOLDG_STAGE3R_CF_E(float, P, 4, false)                \
    TWOLDG_STAGE3R_CF_E(float, P, 2, true)                 \
    TWOLDG_STAGE3R_CF_E(float, P, 4, true)

}  // namespace twoldg
