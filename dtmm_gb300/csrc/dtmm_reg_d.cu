// Register-transform row and column passes, sides 320, 336, 384, 400
// (instantiations; the kernels are in dtmm_regkern.cuh).
#include "dtmm_regkern.cuh"

namespace dtmm {

DTMM_REG_DEFINE(320)
DTMM_REG_DEFINE(336)
DTMM_REG_DEFINE(384)
DTMM_REG_DEFINE(400)

}  // namespace dtmm
