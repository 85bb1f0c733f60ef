// ravu-zoom(-ar) per-frame launches at 16-row tiles.
#include "ravu_zoom_rows.cuh"

namespace pz {
template int launch_zoom_rows<16>(const RavuArgs&, int, int, bool, int, cudaStream_t);
}  // namespace pz
