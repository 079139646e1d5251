// Kernel instantiations for D = 2, P = 3.
#include "ops_impl.cuh"

namespace twoldg {

Ops* make_ops_d2_p3(int prec, const ElementTables<double>& t64, const ElementTables<float>& t32) {
    return make_ops_p<2, 3>(prec, t64, t32);
}

}  // namespace twoldg
