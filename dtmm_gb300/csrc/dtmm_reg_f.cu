// Register-transform row and column passes, sides 512, 1024
// (instantiations; the kernels are in dtmm_regkern.cuh).
#include "dtmm_regkern.cuh"

namespace dtmm {

DTMM_REG_DEFINE(512)
DTMM_REG_DEFINE(1024)

}  // namespace dtmm
