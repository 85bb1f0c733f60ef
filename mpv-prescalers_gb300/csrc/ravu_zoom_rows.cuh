// Per-frame launches of the ravu-zoom(-ar) tile program (ravu_tiles.cuh) at a
// tile height of TR rows: one CTA of 32 x TR threads per 32 x TR block of
// OUTPUT pixels.  Each height is instantiated in its own translation unit
// (ravu_zoom.cu: 8 rows; ravu_zoom_rows4.cu, _rows16.cu).
#pragma once
#include "ravu_tiles.cuh"

namespace pz {

template <typename T, bool H16, int TR>
int launch_zoom_t(const RavuArgs& a, int radius, int cm, bool ar, cudaStream_t s) {
#define PZ_Z(R, CM)                                                     \
  return ar ? launch_tiles<ZoomTile<R, CM, true, T, H16, TR>>(a, s)     \
            : launch_tiles<ZoomTile<R, CM, false, T, H16, TR>>(a, s)
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

// a.lut_h set (fast form): FP16 LUT texels
template <int TR>
int launch_zoom_rows(const RavuArgs& a, int radius, int cm, bool ar, int dtype, cudaStream_t s) {
  if (a.lut_h)
    return dtype == 0 ? launch_zoom_t<float, true, TR>(a, radius, cm, ar, s)
                      : launch_zoom_t<__half, true, TR>(a, radius, cm, ar, s);
  return dtype == 0 ? launch_zoom_t<float, false, TR>(a, radius, cm, ar, s)
                    : launch_zoom_t<__half, false, TR>(a, radius, cm, ar, s);
}

extern template int launch_zoom_rows<4>(const RavuArgs&, int, int, bool, int, cudaStream_t);
extern template int launch_zoom_rows<16>(const RavuArgs&, int, int, bool, int, cudaStream_t);

}  // namespace pz
