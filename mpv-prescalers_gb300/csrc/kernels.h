// Host-side launch interface of the prescaler kernels (internal; the public
// C ABI is include/prescale.h).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace pz {

enum ChMode : int { kLuma = 0, kYuv = 1, kRgb = 2 };

// One RAVU-family dispatch.  Planes are [H][W] with per-plane pitches.
struct RavuArgs {
  const void* in[3];
  int in_pitch[3];
  void* out[3];
  int out_pitch[3];
  int W, H;          // input size
  int OW, OH;        // output size
  const float4* lut;     // [lut_rows][lut_cols] texels
  const float4* lut_ar;  // zoom-ar only
  int lut_rows, lut_cols;
  float ar;
  int32_t* keys;     // optional raw-key output
  int* err;          // device error word (kErr*)
  int staging;       // 0: clamped loads, 1: TMA boxes for interior tiles
  int tile_rows;     // tile height of the per-frame launches: 4, 8 or 16 rows
  float lut_frac;    // zoom LUT bilinear fraction steps (0: exact FP32)
  const uint2* lut_h;  // fast form: the LUT as FP16 texels (4 halves each), or null
  int lut_h_pitch;     // texels per FP16 LUT row (lut_cols rounded up to even)
  int box_w, box_h;    // ravu-zoom TMA staging: the box of this launch's tensor maps (texels x rows)
  float* i11;          // ravu lattice: int11 plane, FP32 [C][H][W] (scratch)
  int i11_half;        // round int11 to FP16 before storing it (the mpv form)
  KeyParams kp;
};

// One NNEDI3 doubling pass.  `xpass` doubles columns, otherwise rows.
struct NnArgs {
  const void* in;
  int in_pitch;
  void* out;
  int out_pitch;
  int W, H;                 // size of the pass input
  int nns, win_h;           // window is 8 x win_h (double_y orientation)
  const float* wts;         // [nns][2][T]: A row then B row per neuron (FP32)
  const float* cs;          // [nns][2]: column sums of A and B
  const float* bias;        // [nns][2]
  const __half* wts_h;      // FP16 packed weights for the tensor-core kernel
  int* err;                 // device error word
};

int launch_lite(const RavuArgs& a, int radius, bool ar, int dtype, cudaStream_t s);
int launch_3x(const RavuArgs& a, int radius, int chmode, int dtype, cudaStream_t s);
int launch_lattice(const RavuArgs& a, int radius, int chmode, int dtype, cudaStream_t s);
int launch_zoom(const RavuArgs& a, int radius, int chmode, bool ar, int dtype, cudaStream_t s);
int launch_nnedi3_simt(const NnArgs& a, bool xpass, int dtype, cudaStream_t s);
int launch_nnedi3_tc(const NnArgs& a, bool xpass, int dtype, cudaStream_t s);
bool nnedi3_tc_supported(int nns, int win_h);
// Neurons per group of the tensor-core weight operand: the host stores B
// chunk-major, NC softmax rows then NC Elliott rows per group.
int nnedi3_tc_chunk(int nns);

}  // namespace pz
