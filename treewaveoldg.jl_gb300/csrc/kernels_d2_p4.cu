// Kernel instantiations for D = 2, P = 4.
#include "ops_impl.cuh"

namespace twoldg {

Ops* make_ops_d2_p4(int prec, const ElementTables<double>& t64, const ElementTables<float>& t32) {
    return make_ops_p<2, 4>(prec, t64, t32);
}

}  // namespace twoldg
