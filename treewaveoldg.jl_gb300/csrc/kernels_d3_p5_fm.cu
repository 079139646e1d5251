// The full-metric stage pass with a compile-time block shape for D = 3, P = 5.
#include "fmstage_r.cuh"

namespace twoldg {

TWOLDG_FMSTAGE_R(5)

}  // namespace twoldg
