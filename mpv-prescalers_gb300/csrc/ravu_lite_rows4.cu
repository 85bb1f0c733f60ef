// ravu-lite(-ar) and ravu-3x per-frame launches at 4-row tiles.
#include "ravu_lite_rows.cuh"

namespace pz {
template int launch_lite_rows<4>(const RavuArgs&, int, bool, int, cudaStream_t);
template int launch_3x_rows<4>(const RavuArgs&, int, int, int, cudaStream_t);
}  // namespace pz
