// Persistent batch kernel, float planes, the fast form's FP16-texel programs.
#include "batch_kernel.cuh"

namespace pz {
PZ_BATCH_DEFINE(f32h, float, true)
}  // namespace pz
