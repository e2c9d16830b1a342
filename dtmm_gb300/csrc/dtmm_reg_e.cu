// Register-transform row and column passes, sides 432, 448, 480
// (instantiations; the kernels are in dtmm_regkern.cuh).
#include "dtmm_regkern.cuh"

namespace dtmm {

DTMM_REG_DEFINE(432)
DTMM_REG_DEFINE(448)
DTMM_REG_DEFINE(480)

}  // namespace dtmm
