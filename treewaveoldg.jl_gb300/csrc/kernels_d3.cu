// Kernel instantiations for D = 3 (one translation unit per dimension so
// that the build compiles them in parallel).
#include "ops_impl.cuh"

namespace twoldg {

Ops* make_ops_d3(int prec, int P, const ElementTables<double>& t64, const ElementTables<float>& t32) {
    return make_ops_dim<3>(prec, P, t64, t32);
}

}  // namespace twoldg
