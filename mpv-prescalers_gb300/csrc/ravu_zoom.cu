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

template <typename T>
PersistentOps zoom_ops(int prog) {
#define PZ_Z(id, R, CM, AR, H) \
  case id: return persistent_ops<ZoomTile<R, CM, AR, T, H>>();
  switch (prog) {
    PZ_Z(kZoom0 + 0, 2, kLuma, false, false) PZ_Z(kZoom0 + 1, 2, kLuma, true, false)
    PZ_Z(kZoom0 + 2, 2, kYuv, false, false) PZ_Z(kZoom0 + 3, 2, kYuv, true, false)
    PZ_Z(kZoom0 + 4, 2, kRgb, false, false) PZ_Z(kZoom0 + 5, 2, kRgb, true, false)
    PZ_Z(kZoom0 + 6, 3, kLuma, false, false) PZ_Z(kZoom0 + 7, 3, kLuma, true, false)
    PZ_Z(kZoom0 + 8, 3, kYuv, false, false) PZ_Z(kZoom0 + 9, 3, kYuv, true, false)
    PZ_Z(kZoom0 + 10, 3, kRgb, false, false) PZ_Z(kZoom0 + 11, 3, kRgb, true, false)
    PZ_Z(kZoomH0 + 0, 2, kLuma, false, true) PZ_Z(kZoomH0 + 1, 2, kLuma, true, true)
    PZ_Z(kZoomH0 + 2, 2, kYuv, false, true) PZ_Z(kZoomH0 + 3, 2, kYuv, true, true)
    PZ_Z(kZoomH0 + 4, 2, kRgb, false, true) PZ_Z(kZoomH0 + 5, 2, kRgb, true, true)
    PZ_Z(kZoomH0 + 6, 3, kLuma, false, true) PZ_Z(kZoomH0 + 7, 3, kLuma, true, true)
    PZ_Z(kZoomH0 + 8, 3, kYuv, false, true) PZ_Z(kZoomH0 + 9, 3, kYuv, true, true)
    PZ_Z(kZoomH0 + 10, 3, kRgb, false, true) PZ_Z(kZoomH0 + 11, 3, kRgb, true, true)
  }
#undef PZ_Z
  return {nullptr, nullptr, nullptr};
}

}  // namespace

PersistentOps persistent_ops_zoom(int prog, int dtype) {
  return dtype == 0 ? zoom_ops<float>(prog) : zoom_ops<__half>(prog);
}

int launch_zoom(const RavuArgs& a, int radius, int cm, bool ar, int dtype, cudaStream_t s) {
  if (a.lut_h)  // fast form: FP16 LUT texels
    return dtype == 0 ? launch_t<float, true>(a, radius, cm, ar, s) : launch_t<__half, true>(a, radius, cm, ar, s);
  return dtype == 0 ? launch_t<float, false>(a, radius, cm, ar, s) : launch_t<__half, false>(a, radius, cm, ar, s);
}

}  // namespace pz
