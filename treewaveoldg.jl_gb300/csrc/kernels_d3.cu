// Kernel instantiations for D = 3 (one translation unit per dimension so
// that the build compiles them in parallel).
#include "ops_impl.cuh"

namespace twoldg {

Ops* make_ops_d3(int prec, int P, const ElementTables<double>& t64, const ElementTables<float>& t32) {
    return make_ops_dim<3>(prec, P, t64, t32);
}

// The full metric's step boundary: t_n += dt for every problem.
__global__ void fm_advance_time_kernel(double* tinfo, int nproblems) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nproblems) tinfo[2 * k] += tinfo[2 * k + 1];
}

void fm_advance_time_launch(double* tinfo, int nproblems, cudaStream_t s) {
    fm_advance_time_kernel<<<(nproblems + 127) / 128, 128, 0, s>>>(tinfo, nproblems);
}

}  // namespace twoldg
