// Internal layout of pz_model (opaque in the public C ABI) and the
// thread-local error setter shared by the entry points.
#pragma once
#include <cuda_fp16.h>

#include "../../include/prescale.h"
#include "kernels.h"

struct pz_model {
  int family = 0, radius = 0, channels = 0;
  float ar = 0.0f;
  float4* d_lut = nullptr;
  float4* d_lut_ar = nullptr;
  float4* d_lut16 = nullptr;     // the LUTs with every value rounded to FP16
  float4* d_lut_ar16 = nullptr;
  __half* d_lut_h = nullptr;     // the LUT as FP16 texels (fast form), rows padded
  int lut_h_pitch = 0;           // to an even texel count (16-byte texel pairs)
  int lut_rows = 0, lut_cols = 0;
  pz::KeyParams kp{};
  int nns = 0, win_w = 0, win_h = 0;
  float* d_wts = nullptr;   // [nns][2][T]
  float* d_cs = nullptr;    // [nns][2]
  float* d_bias = nullptr;  // [nns][2]
  __half* d_wts_h = nullptr;
  int device = 0;
};

namespace pz {
// Record `msg` for pz_last_error() on the calling thread; returns `code`.
int set_error(int code, const char* fmt, ...);

// Device address of the error word the kernels report into (one per device,
// a __device__ variable: nothing is allocated); null if the lookup failed.
// pz_check_device_error reads and clears it.
int* device_error_word();

// pz_run's checks of the options: opts->precision against the plane dtype,
// opts->tile_rows (PZ_OK or PZ_EINVAL with the message set).
int check_opts(const pz_opts* o, int dtype);

// Does the fast form read this model's LUT as FP16 texels?  The lite, 3x and
// zoom programs gather a whole LUT row (or four bilinear texels per block)
// per pixel and are bound by those L1 gathers; FP16 halves them.  The ravu
// lattice reads 5-8 texels per key and keeps FP32, and so does ravu-zoom-ar's
// anti-ringing LUT: most of its values lie below FP16's normal range.
inline bool fast_half_lut(const pz_model* m, int precision) {
  return precision == PZ_PREC_FAST &&
         (m->family == PZ_RAVU_LITE || m->family == PZ_RAVU_3X || m->family == PZ_RAVU_ZOOM);
}

// The LUTs and LUT sampling of a precision form: the mpv form reads the
// FP16-rounded copies and quantises zoom bilinear fractions to 1/256; the
// fast form reads FP16 texels where fast_half_lut says so.
inline void select_lut(const pz_model* m, int precision, RavuArgs* a) {
  const bool mpv = precision == PZ_PREC_MPV;
  a->lut = mpv ? m->d_lut16 : m->d_lut;
  a->lut_ar = mpv ? m->d_lut_ar16 : m->d_lut_ar;
  a->lut_rows = m->lut_rows;
  a->lut_cols = m->lut_cols;
  a->lut_frac = mpv ? 256.0f : 0.0f;
  const bool h = fast_half_lut(m, precision);
  a->lut_h = h ? reinterpret_cast<const uint2*>(m->d_lut_h) : nullptr;
  a->lut_h_pitch = m->lut_h_pitch;
  // the host's int11 texture is rgba16f: the mpv form rounds int11 to FP16,
  // the other forms keep it FP32 between the two lattice launches
  a->i11_half = mpv ? 1 : 0;
}

// Tile height of a model's per-frame launches when the caller asks for none,
// the fastest on GB300 at 480p-1080p (1080p, fast form: 4-row tiles are
// 3-4 % faster than 8 for ravu-r3 / ravu-r4-yuv, 8 % for ravu-3x-r3, even
// for ravu-zoom-ar-r2-rgb; ravu-lite-r2 and ravu-lite-ar-r4 are fastest at
// 8; 16 rows is slower for every program).
inline int default_tile_rows(const pz_model* m) {
  if (m->family == PZ_RAVU_LITE && (m->radius == 2 || (m->radius == 4 && m->ar != 0.0f))) return 8;
  return 4;
}

// Scratch of a ravu lattice chain: the int11 plane, FP32 [channels][H][W].
inline size_t lattice_scratch_bytes(const pz_model* m, int W, int H) {
  return (size_t)(m->channels == PZ_LUMA ? 1 : 3) * W * H * sizeof(float);
}
}  // namespace pz
