// Register-transform row and column passes, sides 128, 144, 160, 192
// (instantiations; the kernels are in dtmm_regkern.cuh).
#include "dtmm_regkern.cuh"

namespace dtmm {

DTMM_REG_DEFINE(128)
DTMM_REG_DEFINE(144)
DTMM_REG_DEFINE(160)
DTMM_REG_DEFINE(192)

}  // namespace dtmm
