// ravu-zoom(-ar) per-frame launches at 4-row tiles.
#include "ravu_zoom_rows.cuh"

namespace pz {
template int launch_zoom_rows<4>(const RavuArgs&, int, int, bool, int, cudaStream_t);
}  // namespace pz
