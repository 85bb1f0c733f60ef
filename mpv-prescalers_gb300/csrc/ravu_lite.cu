// Per-model launches of the ravu-lite(-ar) and ravu-3x tile programs
// (ravu_tiles.cuh): one 256-thread CTA per 32x8 block of input pixels.
#include "ravu_tiles.cuh"

namespace pz {
namespace {

template <typename T, bool H16>
int launch_lite_t(const RavuArgs& a, int radius, bool ar, cudaStream_t s) {
  const int tw = (a.W + kTileW - 1) / kTileW, th = (a.H + kTileH - 1) / kTileH;
#define PZ_LITE(R)                                                      \
  return ar ? launch_tiles<LiteTile<R, true, T, H16>>(a, tw, th, s)     \
            : launch_tiles<LiteTile<R, false, T, H16>>(a, tw, th, s)
  switch (radius) {
    case 2: PZ_LITE(2);
    case 3: PZ_LITE(3);
    case 4: PZ_LITE(4);
  }
#undef PZ_LITE
  return -95;
}

template <typename T, bool H16>
int launch_3x_t(const RavuArgs& a, int radius, int cm, cudaStream_t s) {
  const int tw = (a.W + kTileW - 1) / kTileW, th = (a.H + kTileH - 1) / kTileH;
#define PZ_3X(R)                                                                         \
  return cm == kLuma  ? launch_tiles<ThreeXTile<R, kLuma, T, H16>>(a, tw, th, s)        \
         : cm == kYuv ? launch_tiles<ThreeXTile<R, kYuv, T, H16>>(a, tw, th, s)         \
                      : launch_tiles<ThreeXTile<R, kRgb, T, H16>>(a, tw, th, s)
  switch (radius) {
    case 2: PZ_3X(2);
    case 3: PZ_3X(3);
    case 4: PZ_3X(4);
  }
#undef PZ_3X
  return -95;
}

template <typename T>
PersistentOps lite_ops(int prog) {
#define PZ_L(id, R, AR, H) \
  case id: return persistent_ops<LiteTile<R, AR, T, H>>();
#define PZ_X(id, R, CM, H) \
  case id: return persistent_ops<ThreeXTile<R, CM, T, H>>();
  switch (prog) {
    PZ_L(kLite0 + 0, 2, false, false) PZ_L(kLite0 + 1, 2, true, false) PZ_L(kLite0 + 2, 3, false, false)
    PZ_L(kLite0 + 3, 3, true, false) PZ_L(kLite0 + 4, 4, false, false) PZ_L(kLite0 + 5, 4, true, false)
    PZ_L(kLiteH0 + 0, 2, false, true) PZ_L(kLiteH0 + 1, 2, true, true) PZ_L(kLiteH0 + 2, 3, false, true)
    PZ_L(kLiteH0 + 3, 3, true, true) PZ_L(kLiteH0 + 4, 4, false, true) PZ_L(kLiteH0 + 5, 4, true, true)
    PZ_X(kThreeX0 + 0, 2, kLuma, false) PZ_X(kThreeX0 + 1, 2, kYuv, false) PZ_X(kThreeX0 + 2, 2, kRgb, false)
    PZ_X(kThreeX0 + 3, 3, kLuma, false) PZ_X(kThreeX0 + 4, 3, kYuv, false) PZ_X(kThreeX0 + 5, 3, kRgb, false)
    PZ_X(kThreeX0 + 6, 4, kLuma, false) PZ_X(kThreeX0 + 7, 4, kYuv, false) PZ_X(kThreeX0 + 8, 4, kRgb, false)
    PZ_X(kThreeXH0 + 0, 2, kLuma, true) PZ_X(kThreeXH0 + 1, 2, kYuv, true) PZ_X(kThreeXH0 + 2, 2, kRgb, true)
    PZ_X(kThreeXH0 + 3, 3, kLuma, true) PZ_X(kThreeXH0 + 4, 3, kYuv, true) PZ_X(kThreeXH0 + 5, 3, kRgb, true)
    PZ_X(kThreeXH0 + 6, 4, kLuma, true) PZ_X(kThreeXH0 + 7, 4, kYuv, true) PZ_X(kThreeXH0 + 8, 4, kRgb, true)
  }
#undef PZ_L
#undef PZ_X
  return {nullptr, nullptr, nullptr};
}

}  // namespace

PersistentOps persistent_ops_lite(int prog, int dtype) {
  return dtype == 0 ? lite_ops<float>(prog) : lite_ops<__half>(prog);
}

// a.lut_h set (fast form): the programs read FP16 LUT texels
int launch_lite(const RavuArgs& a, int radius, bool ar, int dtype, cudaStream_t s) {
  if (a.lut_h)
    return dtype == 0 ? launch_lite_t<float, true>(a, radius, ar, s) : launch_lite_t<__half, true>(a, radius, ar, s);
  return dtype == 0 ? launch_lite_t<float, false>(a, radius, ar, s) : launch_lite_t<__half, false>(a, radius, ar, s);
}

int launch_3x(const RavuArgs& a, int radius, int cm, int dtype, cudaStream_t s) {
  if (a.lut_h)
    return dtype == 0 ? launch_3x_t<float, true>(a, radius, cm, s) : launch_3x_t<__half, true>(a, radius, cm, s);
  return dtype == 0 ? launch_3x_t<float, false>(a, radius, cm, s) : launch_3x_t<__half, false>(a, radius, cm, s);
}

}  // namespace pz
