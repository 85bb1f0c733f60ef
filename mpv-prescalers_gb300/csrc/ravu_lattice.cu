// Per-model launches of the ravu lattice chain (ravu_tiles.cuh): the int11
// tile program writes the compact FP32 int11 plane (caller scratch), the
// int10/int01 program reads it and writes every output pixel -- the four
// passes of ravu-r3.hook:15-437 in two launches.
#include "ravu_tiles.cuh"

namespace pz {
namespace {

template <typename T>
int launch_t(const RavuArgs& a, int radius, int cm, cudaStream_t s) {
  const int tw = (a.W + kTileW - 1) / kTileW, th = (a.H + kTileH - 1) / kTileH;
#define PZ_LAT(R, CM)                                     \
  do {                                                    \
    launch_tiles<Int11Tile<R, CM, T>>(a, tw, th, s);      \
    return launch_tiles<LatticeTile<R, CM, T>>(a, tw, th, s); \
  } while (0)
#define PZ_LAT_CM(R)                   \
  if (cm == kLuma) PZ_LAT(R, kLuma);   \
  else if (cm == kYuv) PZ_LAT(R, kYuv); \
  else PZ_LAT(R, kRgb)
  switch (radius) {
    case 2: PZ_LAT_CM(2);
    case 3: PZ_LAT_CM(3);
    case 4: PZ_LAT_CM(4);
  }
#undef PZ_LAT_CM
#undef PZ_LAT
  return -95;
}

template <typename T>
PersistentOps lattice_ops(int prog) {
#define PZ_P(id, Tile, R, CM) \
  case id: return persistent_ops<Tile<R, CM, T>>();
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
  return dtype == 0 ? launch_t<float>(a, radius, cm, s) : launch_t<__half>(a, radius, cm, s);
}

}  // namespace pz
