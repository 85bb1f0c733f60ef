// Per-model launches of the ravu-lite(-ar) and ravu-3x tile programs
// (ravu_tiles.cuh) by tile height, and their persistent batch kernels.
#include "ravu_lite_rows.cuh"

namespace pz {
namespace {

template <typename T>
PersistentOps lite_ops(int prog) {
#define PZ_L(id, R, AR, H) \
  case id: return persistent_ops<LiteTile<R, AR, T, H, kBatchTileRows>>();
#define PZ_X(id, R, CM, H) \
  case id: return persistent_ops<ThreeXTile<R, CM, T, H, kBatchTileRows>>();
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

int launch_lite(const RavuArgs& a, int radius, bool ar, int dtype, cudaStream_t s) {
  switch (a.tile_rows) {
    case 4: return launch_lite_rows<4>(a, radius, ar, dtype, s);
    case 16: return launch_lite_rows<16>(a, radius, ar, dtype, s);
    default: return launch_lite_rows<8>(a, radius, ar, dtype, s);
  }
}

int launch_3x(const RavuArgs& a, int radius, int cm, int dtype, cudaStream_t s) {
  switch (a.tile_rows) {
    case 4: return launch_3x_rows<4>(a, radius, cm, dtype, s);
    case 16: return launch_3x_rows<16>(a, radius, cm, dtype, s);
    default: return launch_3x_rows<8>(a, radius, cm, dtype, s);
  }
}

}  // namespace pz
