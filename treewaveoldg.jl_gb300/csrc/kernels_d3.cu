// Kernel dispatch for D = 3. The instantiations for each order P live in
// their own translation unit (kernels_d3_p<P>.cu) so that the build
// compiles them in parallel.
#include "ops_impl.cuh"

namespace twoldg {

Ops* make_ops_d3_p1(int prec, const ElementTables<double>& t64, const ElementTables<float>& t32);
Ops* make_ops_d3_p2(int prec, const ElementTables<double>& t64, const ElementTables<float>& t32);
Ops* make_ops_d3_p3(int prec, const ElementTables<double>& t64, const ElementTables<float>& t32);
Ops* make_ops_d3_p4(int prec, const ElementTables<double>& t64, const ElementTables<float>& t32);
Ops* make_ops_d3_p5(int prec, const ElementTables<double>& t64, const ElementTables<float>& t32);
Ops* make_ops_d3_p6(int prec, const ElementTables<double>& t64, const ElementTables<float>& t32);
Ops* make_ops_d3_p7(int prec, const ElementTables<double>& t64, const ElementTables<float>& t32);
Ops* make_ops_d3_p8(int prec, const ElementTables<double>& t64, const ElementTables<float>& t32);

Ops* make_ops_d3(int prec, int P, const ElementTables<double>& t64, const ElementTables<float>& t32) {
    switch (P) {
        case 1: return make_ops_d3_p1(prec, t64, t32);
        case 2: return make_ops_d3_p2(prec, t64, t32);
        case 3: return make_ops_d3_p3(prec, t64, t32);
        case 4: return make_ops_d3_p4(prec, t64, t32);
        case 5: return make_ops_d3_p5(prec, t64, t32);
        case 6: return make_ops_d3_p6(prec, t64, t32);
        case 7: return make_ops_d3_p7(prec, t64, t32);
        case 8: return make_ops_d3_p8(prec, t64, t32);
        default: return nullptr;
    }
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
