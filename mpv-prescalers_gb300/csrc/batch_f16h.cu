// Persistent batch kernel, __half planes, the fast form's FP16-texel programs.
#include "batch_kernel.cuh"

namespace pz {
PZ_BATCH_DEFINE(f16h, __half, true)
}  // namespace pz
