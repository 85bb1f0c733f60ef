// ravu-lite(-ar) and ravu-3x per-frame launches at 16-row tiles.
#include "ravu_lite_rows.cuh"

namespace pz {
template int launch_lite_rows<16>(const RavuArgs&, int, bool, int, cudaStream_t);
template int launch_3x_rows<16>(const RavuArgs&, int, int, int, cudaStream_t);
}  // namespace pz
