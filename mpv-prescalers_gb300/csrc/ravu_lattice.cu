// Per-model launches of the ravu lattice chain (ravu_tiles.cuh) by tile
// height, and its persistent batch kernels.
#include "ravu_lattice_rows.cuh"

namespace pz {
namespace {

template <typename T>
PersistentOps lattice_ops(int prog) {
#define PZ_P(id, Tile, R, CM) \
  case id: return persistent_ops<Tile<R, CM, T, kBatchTileRows>>();
  switch (prog) {
    PZ_P(kInt110 + 0, Int11Tile, 2, kLuma) PZ_P(kInt110 + 1, Int11Tile, 2, kYuv) PZ_P(kInt110 + 2, Int11Tile, 2, kRgb)
    PZ_P(kInt110 + 3, Int11Tile, 3, kLuma) PZ_P(kInt110 + 4, Int11Tile, 3, kYuv) PZ_P(kInt110 + 5, Int11Tile, 3, kRgb)
    PZ_P(kInt110 + 6, Int11Tile, 4, kLuma) PZ_P(kInt110 + 7, Int11Tile, 4, kYuv) PZ_P(kInt110 + 8, Int11Tile, 4, kRgb)
    PZ_P(kLattice0 + 0, LatticeTile, 2, kLuma) PZ_P(kLattice0 + 1, LatticeTile, 2, kYuv)
    PZ_P(kLattice0 + 2, LatticeTile, 2, kRgb) PZ_P(kLattice0 + 3, LatticeTile, 3, kLuma)
    PZ_P(kLattice0 + 4, LatticeTile, 3, kYuv) PZ_P(kLattice0 + 5, LatticeTile, 3, kRgb)
    PZ_P(kLattice0 + 6, LatticeTile, 4, kLuma) PZ_P(kLattice0 + 7, LatticeTile, 4, kYuv)
    PZ_P(kLattice0 + 8, LatticeTile, 4, kRgb)
  }
#undef PZ_P
  return {nullptr, nullptr, nullptr};
}

}  // namespace

PersistentOps persistent_ops_lattice(int prog, int dtype) {
  return dtype == 0 ? lattice_ops<float>(prog) : lattice_ops<__half>(prog);
}

int launch_lattice(const RavuArgs& a, int radius, int cm, int dtype, cudaStream_t s) {
  switch (a.tile_rows) {
    case 4: return launch_lattice_rows<4>(a, radius, cm, dtype, s);
    case 16: return launch_lattice_rows<16>(a, radius, cm, dtype, s);
    default: return launch_lattice_rows<8>(a, radius, cm, dtype, s);
  }
}

}  // namespace pz
