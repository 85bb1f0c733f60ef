// Persistent batch kernel, __half planes, FP32-texel programs and the ravu lattice.
#include "batch_kernel.cuh"

namespace pz {
PZ_BATCH_DEFINE(f16, __half, false)
}  // namespace pz
