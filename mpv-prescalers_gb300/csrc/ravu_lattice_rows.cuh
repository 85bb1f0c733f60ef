// Per-frame launches of the ravu lattice chain (ravu_tiles.cuh) at a tile
// height of TR rows: the int11 tile program writes the compact FP32 int11
// plane (caller scratch), the int10/int01 program reads it and writes every
// output pixel -- the four passes of ravu-r3.hook:15-437 in two launches.
// Each height is instantiated in its own translation unit (ravu_lattice.cu:
// 8 rows; ravu_lattice_rows4.cu, _rows16.cu).
#pragma once
#include "ravu_tiles.cuh"

namespace pz {

template <typename T, int TR>
int launch_lattice_t(const RavuArgs& a, int radius, int cm, cudaStream_t s) {
#define PZ_LAT(R, CM)                                                 \
  do {                                                                \
    if (const int rc = launch_tiles<Int11Tile<R, CM, T, TR>>(a, s)) return rc; \
    return launch_tiles<LatticeTile<R, CM, T, TR>>(a, s);             \
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

template <int TR>
int launch_lattice_rows(const RavuArgs& a, int radius, int cm, int dtype, cudaStream_t s) {
  return dtype == 0 ? launch_lattice_t<float, TR>(a, radius, cm, s) : launch_lattice_t<__half, TR>(a, radius, cm, s);
}

extern template int launch_lattice_rows<4>(const RavuArgs&, int, int, int, cudaStream_t);
extern template int launch_lattice_rows<16>(const RavuArgs&, int, int, int, cudaStream_t);

}  // namespace pz
