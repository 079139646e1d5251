// Kernel instantiations for D = 2 (one translation unit per dimension so
// that the build compiles them in parallel).
#include "ops_impl.cuh"

namespace twoldg {

Ops* make_ops_d2(int prec, int P, const ElementTables<double>& t64, const ElementTables<float>& t32) {
    return make_ops_dim<2>(prec, P, t64, t32);
}

}  // namespace twoldg
