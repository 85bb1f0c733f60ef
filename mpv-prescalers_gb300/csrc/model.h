// Internal layout of pz_model (opaque in the public C ABI) and the
// thread-local error setter shared by the entry points.
#pragma once
#include <cuda_fp16.h>

#include "kernels.h"

struct pz_model {
  int family = 0, radius = 0, channels = 0;
  float ar = 0.0f;
  float4* d_lut = nullptr;
  float4* d_lut_ar = nullptr;
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
}  // namespace pz
