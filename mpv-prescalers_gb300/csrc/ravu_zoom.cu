// Per-model launches of the ravu-zoom(-ar) tile program (ravu_tiles.cuh):
// one CTA per 32x8 block of OUTPUT pixels.
#include "ravu_tiles.cuh"

namespace pz {
namespace {

template <typename T, bool H16>
int launch_t(const RavuArgs& a, int radius, int cm, bool ar, cudaStream_t s) {
  const int tw = (a.OW + kTileW - 1) / kTileW, th = (a.OH + kTileH - 1) / kTileH;
#define PZ_Z(R, CM)                                                        \
  return ar ? launch_tiles<ZoomTile<R, CM, true, T, H16>>(a, tw, th, s)    \
            : launch_tiles<ZoomTile<R, CM, false, T, H16>>(a, tw, th, s)
#define PZ_Z_CM(R)                  \
  if (cm == kLuma) PZ_Z(R, kLuma);  \
  else if (cm == kYuv) PZ_Z(R, kYuv); \
  else PZ_Z(R, kRgb)
  switch (radius) {
    case 2: PZ_Z_CM(2);
    case 3: PZ_Z_CM(3);
  }
#undef PZ_Z_CM
#undef PZ_Z
  return -95;
}

}  // namespace

int launch_zoom(const RavuArgs& a, int radius, int cm, bool ar, int dtype, cudaStream_t s) {
  if (a.lut_h)  // fast form: FP16 LUT texels
    return dtype == 0 ? launch_t<float, true>(a, radius, cm, ar, s) : launch_t<__half, true>(a, radius, cm, ar, s);
  return dtype == 0 ? launch_t<float, false>(a, radius, cm, ar, s) : launch_t<__half, false>(a, radius, cm, ar, s);
}

}  // namespace pz
