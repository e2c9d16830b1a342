// Register-transform row and column passes, sides 224, 240, 256, 288
// (instantiations; the kernels are in dtmm_regkern.cuh).
#include "dtmm_regkern.cuh"

namespace dtmm {

DTMM_REG_DEFINE(224)
DTMM_REG_DEFINE(240)
DTMM_REG_DEFINE(256)
DTMM_REG_DEFINE(288)

}  // namespace dtmm
