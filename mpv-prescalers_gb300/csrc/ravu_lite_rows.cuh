// Per-frame launches of the ravu-lite(-ar) and ravu-3x tile programs
// (ravu_tiles.cuh) at a tile height of TR rows: one CTA of 32 x TR threads
// per 32 x TR block of input pixels.  Each height is instantiated in its own
// translation unit (ravu_lite.cu: 8 rows; ravu_lite_rows4.cu, _rows16.cu).
#pragma once
#include "ravu_tiles.cuh"

namespace pz {

template <typename T, bool H16, int TR>
int launch_lite_t(const RavuArgs& a, int radius, bool ar, cudaStream_t s) {
#define PZ_LITE(R)                                                   \
  return ar ? launch_tiles<LiteTile<R, true, T, H16, TR>>(a, s)      \
            : launch_tiles<LiteTile<R, false, T, H16, TR>>(a, s)
  switch (radius) {
    case 2: PZ_LITE(2);
    case 3: PZ_LITE(3);
    case 4: PZ_LITE(4);
  }
#undef PZ_LITE
  return -95;
}

template <typename T, bool H16, int TR>
int launch_3x_t(const RavuArgs& a, int radius, int cm, cudaStream_t s) {
#define PZ_3X(R)                                                                  \
  return cm == kLuma  ? launch_tiles<ThreeXTile<R, kLuma, T, H16, TR>>(a, s)     \
         : cm == kYuv ? launch_tiles<ThreeXTile<R, kYuv, T, H16, TR>>(a, s)      \
                      : launch_tiles<ThreeXTile<R, kRgb, T, H16, TR>>(a, s)
  switch (radius) {
    case 2: PZ_3X(2);
    case 3: PZ_3X(3);
    case 4: PZ_3X(4);
  }
#undef PZ_3X
  return -95;
}

// a.lut_h set (fast form): the programs read FP16 LUT texels
template <int TR>
int launch_lite_rows(const RavuArgs& a, int radius, bool ar, int dtype, cudaStream_t s) {
  if (a.lut_h)
    return dtype == 0 ? launch_lite_t<float, true, TR>(a, radius, ar, s)
                      : launch_lite_t<__half, true, TR>(a, radius, ar, s);
  return dtype == 0 ? launch_lite_t<float, false, TR>(a, radius, ar, s)
                    : launch_lite_t<__half, false, TR>(a, radius, ar, s);
}

template <int TR>
int launch_3x_rows(const RavuArgs& a, int radius, int cm, int dtype, cudaStream_t s) {
  if (a.lut_h)
    return dtype == 0 ? launch_3x_t<float, true, TR>(a, radius, cm, s) : launch_3x_t<__half, true, TR>(a, radius, cm, s);
  return dtype == 0 ? launch_3x_t<float, false, TR>(a, radius, cm, s) : launch_3x_t<__half, false, TR>(a, radius, cm, s);
}

extern template int launch_lite_rows<4>(const RavuArgs&, int, bool, int, cudaStream_t);
extern template int launch_lite_rows<16>(const RavuArgs&, int, bool, int, cudaStream_t);
extern template int launch_3x_rows<4>(const RavuArgs&, int, int, int, cudaStream_t);
extern template int launch_3x_rows<16>(const RavuArgs&, int, int, int, cudaStream_t);

}  // namespace pz
