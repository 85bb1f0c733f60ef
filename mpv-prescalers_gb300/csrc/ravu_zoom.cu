// Per-model launches of the ravu-zoom(-ar) tile program (ravu_tiles.cuh) by
// tile height, and its persistent batch kernels.
#include "ravu_zoom_rows.cuh"

namespace pz {
namespace {

template <typename T>
PersistentOps zoom_ops(int prog) {
#define PZ_Z(id, R, CM, AR, H) \
  case id: return persistent_ops<ZoomTile<R, CM, AR, T, H, kBatchTileRows>>();
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
  switch (a.tile_rows) {
    case 4: return launch_zoom_rows<4>(a, radius, cm, ar, dtype, s);
    case 16: return launch_zoom_rows<16>(a, radius, cm, ar, dtype, s);
    default: return launch_zoom_rows<8>(a, radius, cm, ar, dtype, s);
  }
}

}  // namespace pz
