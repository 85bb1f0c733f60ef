// Per-model launches of the ravu lattice chain (ravu_tiles.cuh): the int11
// tile program, then the int10/int01 program, which reads int11 back from
// the output plane -- the four passes of ravu-r3.hook:15-437 in two launches
// with no intermediate plane outside the output.
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

}  // namespace

int launch_lattice(const RavuArgs& a, int radius, int cm, int dtype, cudaStream_t s) {
  return dtype == 0 ? launch_t<float>(a, radius, cm, s) : launch_t<__half>(a, radius, cm, s);
}

}  // namespace pz
