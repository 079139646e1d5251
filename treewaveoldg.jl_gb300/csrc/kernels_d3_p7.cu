// Kernel instantiations for D = 3, P = 7.
#include "ops_impl.cuh"

namespace twoldg {

Ops* make_ops_d3_p7(int prec, const ElementTables<double>& t64, const ElementTables<float>& t32) {
    return make_ops_p<3, 7>(prec, t64, t32);
}

}  // namespace twoldg
