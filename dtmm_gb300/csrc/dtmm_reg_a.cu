// Register-transform row and column passes, sides 64, 80, 96, 112
// (instantiations; the kernels are in dtmm_regkern.cuh).
#include "dtmm_regkern.cuh"

namespace dtmm {

DTMM_REG_DEFINE(64)
DTMM_REG_DEFINE(80)
DTMM_REG_DEFINE(96)
DTMM_REG_DEFINE(112)

}  // namespace dtmm
