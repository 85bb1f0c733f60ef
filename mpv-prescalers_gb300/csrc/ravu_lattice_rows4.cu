// ravu lattice chain per-frame launches at 4-row tiles.
#include "ravu_lattice_rows.cuh"

namespace pz {
template int launch_lattice_rows<4>(const RavuArgs&, int, int, int, cudaStream_t);
}  // namespace pz
