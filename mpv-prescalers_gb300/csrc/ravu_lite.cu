// ravu-lite(-ar) 2x and ravu-3x 3x: one thread per input pixel.
//
// Reference: compute/ravu-lite-ar-r3.hook:15-171 (tile + halo in shared
// memory, one key and four sub-pixel dot products per input pixel, the
// anti-ringing clamp, four stores), root form ravu-lite-r3.hook:15-131;
// compute/ravu-3x-r2.hook:15-115 (eight keyed outputs + the centre copy).
//
// GB300 mapping: a 32x8 block covers 32x8 input pixels; its (32+n-1) x
// (8+n-1) window tile is staged in shared memory with clamp-to-edge reads
// (the border mode of the mpv textures).  The LUT row of each pixel's key is
// read as float4 texels through the read-only path (L1/L2 resident: 23-173
// KB).  Outputs leave as 2-wide vector stores, so a warp writes 2 x 256 B of
// contiguous output rows.
#include "kernels.h"

namespace pz {
namespace {

// Stage the (TW x TH) clamp-to-edge window tile of one plane.
template <int TW, int TH, typename T>
__device__ __forceinline__ void stage_tile(float (*tile)[TW], const T* in, int pitch, int W, int H,
                                           int x0, int y0) {
  for (int i = threadIdx.y * blockDim.x + threadIdx.x; i < TW * TH; i += blockDim.x * blockDim.y) {
    int ty = i / TW, tx = i % TW;
    int gx = clampi(x0 + tx, 0, W - 1);
    int gy = clampi(y0 + ty, 0, H - 1);
    tile[ty][tx] = ldp(in + (size_t)gy * pitch + gx);
  }
}

// Does lite LUT column c take part in the anti-ringing sums?  r2: every
// tap; r3/r4: the 13-tap diamond |dx|+|dy| <= 2 (ravu-lite-ar-r3.hook:93-170).
__host__ __device__ constexpr int cabs(int v) { return v < 0 ? -v : v; }
template <int R>
__host__ __device__ constexpr bool lite_ar_col(int c) {
  return R == 2 || cabs(c / (2 * R - 1) - (R - 1)) + cabs(c % (2 * R - 1) - (R - 1)) <= 2;
}

template <int R, bool AR, typename T>
__global__ void __launch_bounds__(256) lite_kernel(const __grid_constant__ RavuArgs p) {
  constexpr int N = 2 * R - 1, S = N * N, HALO = R - 1;
  constexpr int TW = 32 + N - 1, TH = 8 + N - 1;
  __shared__ float tile[TH][TW];
  // anti-ringing powers of every tile value, computed once per value instead
  // of once per window tap: (h32, l32, h33, l33)
  __shared__ float4 ptile[AR ? TH : 1][AR ? TW : 1];
  const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 8;
  stage_tile<TW, TH>(tile, static_cast<const T*>(p.in[0]), p.in_pitch[0], p.W, p.H, x0 - HALO, y0 - HALO);
  __syncthreads();
  if (AR) {
    for (int i = threadIdx.y * 32 + threadIdx.x; i < TW * TH; i += 256) {
      const ArPow q = ar_pow(tile[i / TW][i % TW]);
      ptile[i / TW][i % TW] = make_float4(q.h32, q.l32, q.h33, q.l33);
    }
    __syncthreads();
  }
  const int gx = x0 + threadIdx.x, gy = y0 + threadIdx.y;
  if (gx >= p.W || gy >= p.H) return;
  const int tx = threadIdx.x, ty = threadIdx.y;
  auto get = [&](int kx, int ky) { return tile[ty + ky][tx + kx]; };
  auto pw = [&](int k) {
    const float4 q = ptile[AR ? ty + k % N : 0][AR ? tx + k / N : 0];
    return ArPow{q.x, q.z, q.y, q.w};
  };
  float a, b, d;
  structure_tensor<N, false>(get, p.kp, a, b, d);
  int key = ravu_key(a, b, d, p.kp);
  if (p.keys) p.keys[(size_t)gy * p.W + gx] = key;
  const float4* L = p.lut + (size_t)min(max(key, 0), p.lut_rows - 1) * p.lut_cols;
  float4 res = make_float4(0.f, 0.f, 0.f, 0.f);
  float4 hi = res, lo = res, hi2 = res, lo2 = res;
#pragma unroll
  for (int c = 0; c < S / 2; c++) {
    float4 w = __ldg(L + c);
    float va = get(c / N, c % N), vb = get((S - 1 - c) / N, (S - 1 - c) % N);
    // res += va * w + vb * w.wzyx
    res.x += va * w.x + vb * w.w;
    res.y += va * w.y + vb * w.z;
    res.z += va * w.z + vb * w.y;
    res.w += va * w.w + vb * w.x;
    if (AR && lite_ar_col<R>(c)) {
      float4 wg = make_float4(fmaxf(w.x, 0.f), fmaxf(w.y, 0.f), fmaxf(w.z, 0.f), fmaxf(w.w, 0.f));
      const ArPow pa = pw(c), pb = pw(S - 1 - c);
      hi.x += pa.h32 * wg.x + pb.h32 * wg.w;  hi.y += pa.h32 * wg.y + pb.h32 * wg.z;
      hi.z += pa.h32 * wg.z + pb.h32 * wg.y;  hi.w += pa.h32 * wg.w + pb.h32 * wg.x;
      lo.x += pa.l32 * wg.x + pb.l32 * wg.w;  lo.y += pa.l32 * wg.y + pb.l32 * wg.z;
      lo.z += pa.l32 * wg.z + pb.l32 * wg.y;  lo.w += pa.l32 * wg.w + pb.l32 * wg.x;
      hi2.x += pa.h33 * wg.x + pb.h33 * wg.w; hi2.y += pa.h33 * wg.y + pb.h33 * wg.z;
      hi2.z += pa.h33 * wg.z + pb.h33 * wg.y; hi2.w += pa.h33 * wg.w + pb.h33 * wg.x;
      lo2.x += pa.l33 * wg.x + pb.l33 * wg.w; lo2.y += pa.l33 * wg.y + pb.l33 * wg.z;
      lo2.z += pa.l33 * wg.z + pb.l33 * wg.y; lo2.w += pa.l33 * wg.w + pb.l33 * wg.x;
    }
  }
  {
    constexpr int c = S / 2;
    float4 w = __ldg(L + c);
    float v = get(c / N, c % N);
    res.x += v * w.x; res.y += v * w.y; res.z += v * w.z; res.w += v * w.w;
    if (AR) {
      float4 wg = make_float4(fmaxf(w.x, 0.f), fmaxf(w.y, 0.f), fmaxf(w.z, 0.f), fmaxf(w.w, 0.f));
      const ArPow pc = pw(c);
      hi.x += pc.h32 * wg.x; hi.y += pc.h32 * wg.y; hi.z += pc.h32 * wg.z; hi.w += pc.h32 * wg.w;
      lo.x += pc.l32 * wg.x; lo.y += pc.l32 * wg.y; lo.z += pc.l32 * wg.z; lo.w += pc.l32 * wg.w;
      hi2.x += pc.h33 * wg.x; hi2.y += pc.h33 * wg.y; hi2.z += pc.h33 * wg.z; hi2.w += pc.h33 * wg.w;
      lo2.x += pc.l33 * wg.x; lo2.y += pc.l33 * wg.y; lo2.z += pc.l33 * wg.z; lo2.w += pc.l33 * wg.w;
    }
  }
  if (AR) {  // no [0,1] clamp after anti-ringing (compute/ravu-lite-ar-r3.hook:166)
    res.x = ar_finish(res.x, lo.x, hi.x, lo2.x, hi2.x, p.ar);
    res.y = ar_finish(res.y, lo.y, hi.y, lo2.y, hi2.y, p.ar);
    res.z = ar_finish(res.z, lo.z, hi.z, lo2.z, hi2.z, p.ar);
    res.w = ar_finish(res.w, lo.w, hi.w, lo2.w, hi2.w, p.ar);
  } else {
    res.x = clampf(res.x, 0.f, 1.f); res.y = clampf(res.y, 0.f, 1.f);
    res.z = clampf(res.z, 0.f, 1.f); res.w = clampf(res.w, 0.f, 1.f);
  }
  // res[0..3] -> offsets (0,0), (0,1), (1,0), (1,1)  (compute/ravu-lite-r3.hook:101-104)
  T* out = static_cast<T*>(p.out[0]);
  const int op = p.out_pitch[0];
  stp2(out + (size_t)(2 * gy) * op + 2 * gx, res.x, res.z);
  stp2(out + (size_t)(2 * gy + 1) * op + 2 * gx, res.y, res.w);
}

// ------------------------------------------------------------------ 3x ----
template <int R, int CM, typename T>
__global__ void __launch_bounds__(256) three_x_kernel(const __grid_constant__ RavuArgs p) {
  constexpr int N = 2 * R - 1, S = N * N, HALO = R - 1;
  constexpr int TW = 32 + N - 1, TH = 8 + N - 1;
  constexpr int C = CM == kLuma ? 1 : 3;
  __shared__ float tile[C][TH][TW];
  __shared__ float ltile[CM == kRgb ? TH : 1][CM == kRgb ? TW : 1];
  const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 8;
#pragma unroll
  for (int c = 0; c < C; c++)
    stage_tile<TW, TH>(tile[c], static_cast<const T*>(p.in[c]), p.in_pitch[c], p.W, p.H, x0 - HALO, y0 - HALO);
  __syncthreads();
  if (CM == kRgb) {
    for (int i = threadIdx.y * 32 + threadIdx.x; i < TW * TH; i += 256) {
      int ty = i / TW, tx = i % TW;
      ltile[ty][tx] = rgb_luma(tile[0][ty][tx], tile[1][ty][tx], tile[2][ty][tx]);
    }
    __syncthreads();
  }
  const int gx = x0 + threadIdx.x, gy = y0 + threadIdx.y;
  if (gx >= p.W || gy >= p.H) return;
  const int tx = threadIdx.x, ty = threadIdx.y;
  auto lum = [&](int kx, int ky) { return CM == kRgb ? ltile[ty + ky][tx + kx] : tile[0][ty + ky][tx + kx]; };
  float a, b, d;
  structure_tensor<N, false>(lum, p.kp, a, b, d);
  int key = ravu_key(a, b, d, p.kp);
  if (p.keys) p.keys[(size_t)gy * p.W + gx] = key;
  const float4* L = p.lut + (size_t)min(max(key, 0), p.lut_rows - 1) * p.lut_cols;
  float4 r0[C], r1[C];
#pragma unroll
  for (int c = 0; c < C; c++) {
    r0[c] = make_float4(0.f, 0.f, 0.f, 0.f);
    r1[c] = r0[c];
  }
#pragma unroll
  for (int t = 0; t < S / 2; t++) {
    float4 w0 = __ldg(L + 2 * t), w1 = __ldg(L + 2 * t + 1);
#pragma unroll
    for (int c = 0; c < C; c++) {
      float va = tile[c][ty + t % N][tx + t / N];
      float vb = tile[c][ty + (S - 1 - t) % N][tx + (S - 1 - t) / N];
      // res0 += a*w0 + b*w1.wzyx; res1 += a*w1 + b*w0.wzyx
      r0[c].x += va * w0.x + vb * w1.w; r0[c].y += va * w0.y + vb * w1.z;
      r0[c].z += va * w0.z + vb * w1.y; r0[c].w += va * w0.w + vb * w1.x;
      r1[c].x += va * w1.x + vb * w0.w; r1[c].y += va * w1.y + vb * w0.z;
      r1[c].z += va * w1.z + vb * w0.y; r1[c].w += va * w1.w + vb * w0.x;
    }
  }
  constexpr int tc = S / 2;
  float4 w0 = __ldg(L + 2 * tc), w1 = __ldg(L + 2 * tc + 1);
#pragma unroll
  for (int c = 0; c < C; c++) {
    float v = tile[c][ty + tc % N][tx + tc / N];
    r0[c].x += v * w0.x; r0[c].y += v * w0.y; r0[c].z += v * w0.z; r0[c].w += v * w0.w;
    r1[c].x += v * w1.x; r1[c].y += v * w1.y; r1[c].z += v * w1.z; r1[c].w += v * w1.w;
    float4 a0 = make_float4(clampf(r0[c].x, 0.f, 1.f), clampf(r0[c].y, 0.f, 1.f), clampf(r0[c].z, 0.f, 1.f),
                            clampf(r0[c].w, 0.f, 1.f));
    float4 a1 = make_float4(clampf(r1[c].x, 0.f, 1.f), clampf(r1[c].y, 0.f, 1.f), clampf(r1[c].z, 0.f, 1.f),
                            clampf(r1[c].w, 0.f, 1.f));
    // imageStore(gid*3 + (dx,dy)): res0 -> (0,0),(0,1),(0,2),(1,0); centre (1,1);
    // res1 -> (1,2),(2,0),(2,1),(2,2)   (compute/ravu-3x-r2.hook:106-114)
    T* o = static_cast<T*>(p.out[c]);
    const size_t op = p.out_pitch[c];
    T* r = o + (size_t)(3 * gy) * op + 3 * gx;
    stp(r, a0.x); stp(r + 1, a0.w); stp(r + 2, a1.y);
    r += op;
    stp(r, a0.y); stp(r + 1, v); stp(r + 2, a1.z);
    r += op;
    stp(r, a0.z); stp(r + 1, a1.x); stp(r + 2, a1.w);
  }
}

template <typename T>
int launch_lite_t(const RavuArgs& a, int radius, bool ar, cudaStream_t s) {
  dim3 blk(32, 8), grd((a.W + 31) / 32, (a.H + 7) / 8);
#define PZ_LITE(R, A) lite_kernel<R, A, T><<<grd, blk, 0, s>>>(a)
  if (radius == 2) { if (ar) PZ_LITE(2, true); else PZ_LITE(2, false); }
  else if (radius == 3) { if (ar) PZ_LITE(3, true); else PZ_LITE(3, false); }
  else if (radius == 4) { if (ar) PZ_LITE(4, true); else PZ_LITE(4, false); }
  else return -95;
#undef PZ_LITE
  return 0;
}

template <typename T>
int launch_3x_t(const RavuArgs& a, int radius, int cm, cudaStream_t s) {
  dim3 blk(32, 8), grd((a.W + 31) / 32, (a.H + 7) / 8);
#define PZ_3X(R)                                                         \
  if (cm == kLuma) three_x_kernel<R, kLuma, T><<<grd, blk, 0, s>>>(a);   \
  else if (cm == kYuv) three_x_kernel<R, kYuv, T><<<grd, blk, 0, s>>>(a); \
  else three_x_kernel<R, kRgb, T><<<grd, blk, 0, s>>>(a)
  if (radius == 2) { PZ_3X(2); }
  else if (radius == 3) { PZ_3X(3); }
  else if (radius == 4) { PZ_3X(4); }
  else return -95;
#undef PZ_3X
  return 0;
}

}  // namespace

int launch_lite(const RavuArgs& a, int radius, bool ar, int dtype, cudaStream_t s) {
  return dtype == 0 ? launch_lite_t<float>(a, radius, ar, s) : launch_lite_t<__half>(a, radius, ar, s);
}

int launch_3x(const RavuArgs& a, int radius, int cm, int dtype, cudaStream_t s) {
  return dtype == 0 ? launch_3x_t<float>(a, radius, cm, s) : launch_3x_t<__half>(a, radius, cm, s);
}

}  // namespace pz
