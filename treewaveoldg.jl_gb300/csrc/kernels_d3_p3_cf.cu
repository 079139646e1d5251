// The register-line stage with its coarse-fine prologue for D = 3, P = 3.
#include "stage3r_cf.cuh"

namespace twoldg {

TWOLDG_STAGE3R_CF(3)

}  // namespace twoldg
