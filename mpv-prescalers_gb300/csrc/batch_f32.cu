// Persistent batch kernel, float planes, FP32-texel programs and the ravu lattice.
#include "batch_kernel.cuh"

namespace pz {
PZ_BATCH_DEFINE(f32, float, false)
}  // namespace pz
