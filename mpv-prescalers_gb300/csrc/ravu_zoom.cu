// ravu-zoom(-ar) arbitrary-ratio upscale: one thread per OUTPUT pixel.
//
// Reference: ravu-zoom-r2.hook:15-139 and compute/ravu-zoom-ar-r2-rgb.hook:
// 15-238.  Output pixel (X, Y) maps to input position
// pos = (X + 0.5) * W / OW (centre-aligned, //!OFFSET ALIGN); the window is
// anchored at floor(pos - 0.5) and subpix = fract(pos - 0.5) selects a point
// inside the key's 9x9 block of the LUT (//!FILTER LINEAR, LUTPOS(x, 9)).
// The mirrored half of the taps reads the LUT at 1 - subpix.
//
// GB300 mapping: a 32x8 block of output pixels stages the input rectangle it
// touches (at most (32+n+1) x (8+n+1) for upscaling) in shared memory.  The
// position arithmetic is exact integer math: the window anchor and subpix
// come from ((2X+1) W - OW) / (2 OW), so only the final FP32 rounding of the
// fraction remains.  LUT texels are blended in FP32 (exact bilinear) from
// the read-only path; the LUTs (746 KB, 1.87 MB) stay L2 resident.
#include "kernels.h"

namespace pz {
namespace {

struct Pos {
  int i;     // floor(pos - 0.5)
  float s;   // fract(pos - 0.5)
};

__device__ __forceinline__ Pos out_to_in(int X, int W, int OW) {
  long long num = (2LL * X + 1) * W - OW;  // (pos - 0.5) * 2 OW
  long long den = 2LL * OW;
  long long q = num >= 0 ? num / den : -((-num + den - 1) / den);
  return {(int)q, (float)(num - q * den) / (float)den};
}

// Bilinear fetch of one LUT texel at block column `blk`, sub-position (sx, sy)
// inside key row block `key` (texel x = blk*9 + 8 sx, y = key*9 + 8 sy).
__device__ __forceinline__ float4 lut_bilinear(const float4* lut, int rows, int cols, int key, int blk,
                                               float sx, float sy) {
  float fx8 = 8.0f * sx, fy8 = 8.0f * sy;
  float x0f = floorf(fx8), y0f = floorf(fy8);
  float fx = fx8 - x0f, fy = fy8 - y0f;
  int xa = min(blk * 9 + (int)x0f, cols - 1), xb = min(xa + 1, cols - 1);
  int ya = clampi(key * 9 + (int)y0f, 0, rows - 1), yb = min(ya + 1, rows - 1);
  float4 v00 = __ldg(lut + (size_t)ya * cols + xa), v01 = __ldg(lut + (size_t)ya * cols + xb);
  float4 v10 = __ldg(lut + (size_t)yb * cols + xa), v11 = __ldg(lut + (size_t)yb * cols + xb);
  float gx = 1.0f - fx, gy = 1.0f - fy;
  float4 r;
  r.x = (v00.x * gx + v01.x * fx) * gy + (v10.x * gx + v11.x * fx) * fy;
  r.y = (v00.y * gx + v01.y * fx) * gy + (v10.y * gx + v11.y * fx) * fy;
  r.z = (v00.z * gx + v01.z * fx) * gy + (v10.z * gx + v11.z * fx) * fy;
  r.w = (v00.w * gx + v01.w * fx) * gy + (v10.w * gx + v11.w * fx) * fy;
  return r;
}

__device__ __forceinline__ float comp(const float4& v, int i) {
  return i == 0 ? v.x : (i == 1 ? v.y : (i == 2 ? v.z : v.w));
}

template <int R, int CM, bool AR, typename T>
__global__ void __launch_bounds__(256) zoom_kernel(const __grid_constant__ RavuArgs p, int* err) {
  constexpr int N = 2 * R, S = N * N, LO = R - 1;
  constexpr int RW = 32 + N + 1, RH = 8 + N + 1;
  constexpr int C = CM == kLuma ? 1 : 3;
  constexpr int NB = (S / 2 + 3) / 4;  // LUT texels per half window
  __shared__ float tile[C][RH][RW];
  __shared__ float ltile[RH][RW];
  const int X0 = blockIdx.x * 32, Y0 = blockIdx.y * 8;
  const int X1 = min(X0 + 31, p.OW - 1), Y1 = min(Y0 + 7, p.OH - 1);
  const int rx = out_to_in(X0, p.W, p.OW).i - LO, ry = out_to_in(Y0, p.H, p.OH).i - LO;
  const int rw = out_to_in(X1, p.W, p.OW).i + R - rx + 1, rh = out_to_in(Y1, p.H, p.OH).i + R - ry + 1;
  if (rw > RW || rh > RH) {  // only reachable when downscaling, which the host rejects
    if (threadIdx.x == 0 && threadIdx.y == 0) atomicCAS(err, 0, kErrTileOverflow);
    return;
  }
  for (int i = threadIdx.y * 32 + threadIdx.x; i < rw * rh; i += 256) {
    int ty = i / rw, tx = i % rw;
    int gx = clampi(rx + tx, 0, p.W - 1), gy = clampi(ry + ty, 0, p.H - 1);
    float v[3];
#pragma unroll
    for (int c = 0; c < C; c++) {
      v[c] = ldp(static_cast<const T*>(p.in[c]) + (size_t)gy * p.in_pitch[c] + gx);
      tile[c][ty][tx] = v[c];
    }
    ltile[ty][tx] = CM == kRgb ? rgb_luma(v[0], v[1], v[2]) : v[0];
  }
  __syncthreads();
  const int X = X0 + threadIdx.x, Y = Y0 + threadIdx.y;
  if (X >= p.OW || Y >= p.OH) return;
  const Pos px = out_to_in(X, p.W, p.OW), py = out_to_in(Y, p.H, p.OH);
  const int bx = px.i - LO - rx, by = py.i - LO - ry;  // window origin in the tile
  auto lum = [&](int kx, int ky) { return ltile[by + ky][bx + kx]; };
  float a, b, d;
  structure_tensor<N, true>(lum, p.kp, a, b, d);
  const int key = ravu_key(a, b, d, p.kp);  // no +0.5 row centring (ravu-zoom-r2.hook:124)
  if (p.keys) p.keys[(size_t)Y * p.OW + X] = key;
  const float sx = px.s, sy = py.s, ix = 1.0f - sx, iy = 1.0f - sy;
  float res[C], hi[C], lo[C], hi2[C], lo2[C];
#pragma unroll
  for (int c = 0; c < C; c++) res[c] = hi[c] = lo[c] = hi2[c] = lo2[c] = 0.0f;
#pragma unroll
  for (int blk = 0; blk < NB; blk++) {
    const float4 ws = lut_bilinear(p.lut, p.lut_rows, p.lut_cols, key, blk, sx, sy);
    const float4 wi = lut_bilinear(p.lut, p.lut_rows, p.lut_cols, key, blk, ix, iy);
    float4 as, ai;
    if (AR) {
      as = lut_bilinear(p.lut_ar, p.lut_rows, p.lut_cols, key, blk, sx, sy);
      ai = lut_bilinear(p.lut_ar, p.lut_rows, p.lut_cols, key, blk, ix, iy);
    }
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int i = blk * 4 + j;
      if (i < S / 2) {
        const int k2 = S - 1 - i;
#pragma unroll
        for (int c = 0; c < C; c++) {
          const float va = tile[c][by + i % N][bx + i / N];
          const float vb = tile[c][by + k2 % N][bx + k2 / N];
          res[c] += va * comp(ws, j);
          res[c] += vb * comp(wi, j);
          if (AR) {
            ArPow pa = ar_pow(va), pb = ar_pow(vb);
            const float wa = comp(as, j), wb = comp(ai, j);
            hi[c] += pa.h32 * wa + pb.h32 * wb;
            lo[c] += pa.l32 * wa + pb.l32 * wb;
            hi2[c] += pa.h33 * wa + pb.h33 * wb;
            lo2[c] += pa.l33 * wa + pb.l33 * wb;
          }
        }
      }
    }
  }
#pragma unroll
  for (int c = 0; c < C; c++) {
    float v = AR ? ar_finish(res[c], lo[c], hi[c], lo2[c], hi2[c], p.ar) : clampf(res[c], 0.f, 1.f);
    stp(static_cast<T*>(p.out[c]) + (size_t)Y * p.out_pitch[c] + X, v);
  }
}

template <typename T>
int launch_t(const RavuArgs& a, int radius, int cm, bool ar, int* err, cudaStream_t s) {
  dim3 blk(32, 8), grd((a.OW + 31) / 32, (a.OH + 7) / 8);
#define PZ_Z(R, CM)                                                  \
  if (ar) zoom_kernel<R, CM, true, T><<<grd, blk, 0, s>>>(a, err);   \
  else zoom_kernel<R, CM, false, T><<<grd, blk, 0, s>>>(a, err)
#define PZ_Z_CM(R)                  \
  if (cm == kLuma) { PZ_Z(R, kLuma); } \
  else if (cm == kYuv) { PZ_Z(R, kYuv); } \
  else { PZ_Z(R, kRgb); }
  if (radius == 2) { PZ_Z_CM(2); }
  else if (radius == 3) { PZ_Z_CM(3); }
  else return -95;
#undef PZ_Z_CM
#undef PZ_Z
  return 0;
}

}  // namespace

int* device_error_word();

int launch_zoom(const RavuArgs& a, int radius, int cm, bool ar, int dtype, cudaStream_t s) {
  int* err = device_error_word();
  if (!err) return -5;
  return dtype == 0 ? launch_t<float>(a, radius, cm, ar, err, s) : launch_t<__half>(a, radius, cm, ar, err, s);
}

}  // namespace pz
