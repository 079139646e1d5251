// Kernel instantiations for D = 3, P = 8.
#include "ops_impl.cuh"

namespace twoldg {

Ops* make_ops_d3_p8(int prec, const ElementTables<double>& t64, const ElementTables<float>& t32) {
    return make_ops_p<3, 8>(prec, t64, t32);
}

}  // namespace twoldg
