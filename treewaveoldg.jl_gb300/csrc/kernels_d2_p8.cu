// Kernel instantiations for D = 2, P = 8.
#include "ops_impl.cuh"

namespace twoldg {

Ops* make_ops_d2_p8(int prec, const ElementTables<double>& t64, const ElementTables<float>& t32) {
    return make_ops_p<2, 8>(prec, t64, t32);
}

}  // namespace twoldg
