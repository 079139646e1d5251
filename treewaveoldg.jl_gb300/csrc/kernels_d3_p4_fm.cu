// The full-metric stage pass with a compile-time block shape for D = 3, P = 4.
#include "fmstage_r.cuh"

namespace twoldg {

TWOLDG_FMSTAGE_R(4)

}  // namespace twoldg
