// ravu (luma / yuv / rgb) 2x: the four-pass lattice chain in two kernels.
//
// Reference: ravu-r3.hook:15-437 (int11, int10, int01, combine) and its
// compute form compute/ravu-r3.hook:15-430 (int11, then int10 + int01 +
// copies).  Output pixel (2i, 2j) is the input, (2i+1, 2j+1) = int11 (the
// diagonal half-pixel), (2i+1, 2j) = int10 and (2i, 2j+1) = int01, which are
// keyed filters on the 45-degree lattice interleaving input and int11 pixels.
//
// GB300 mapping: kernel A computes int11 and writes it, together with the
// input copy, straight into its final place in the output plane; kernel B
// stages the input tile and the int11 tile (read back from the output at
// clamped int11 coordinates, which is the clamp-to-edge of the int11
// texture) and evaluates both lattice filters per thread.  No intermediate
// plane exists outside the output.
#include "kernels.h"

namespace pz {
namespace {

// Stage the clamp-to-edge tiles of all planes; RGB also gets a Rec.709 luma
// tile (yuv and luma read their key input from plane 0 directly).
template <int CM, typename T, int TW, int TH, int LH, int LW>
__device__ __forceinline__ void stage_planes(float (*tile)[TH][TW], float (*ltile)[LW], const RavuArgs& p,
                                             int x0, int y0) {
  constexpr int C = CM == kLuma ? 1 : 3;
  for (int i = threadIdx.y * 32 + threadIdx.x; i < TW * TH; i += 256) {
    int ty = i / TW, tx = i % TW;
    int gx = clampi(x0 + tx, 0, p.W - 1), gy = clampi(y0 + ty, 0, p.H - 1);
    float v[3];
#pragma unroll
    for (int c = 0; c < C; c++) {
      v[c] = ldp(static_cast<const T*>(p.in[c]) + (size_t)gy * p.in_pitch[c] + gx);
      tile[c][ty][tx] = v[c];
    }
    if (CM == kRgb) ltile[ty][tx] = rgb_luma(v[0], v[1], v[2]);
  }
}

// int11 pass: the keyed filter over the input window (ravu-r3.hook:15-146).
template <int R, int CM, typename T>
__global__ void __launch_bounds__(256) int11_kernel(const __grid_constant__ RavuArgs p) {
  constexpr int N = 2 * R, S = N * N, HALO = R - 1;
  constexpr int TW = 32 + N - 1, TH = 8 + N - 1;
  constexpr int C = CM == kLuma ? 1 : 3;
  constexpr int LH = CM == kRgb ? TH : 1, LW = CM == kRgb ? TW : 1;
  __shared__ float tile[C][TH][TW];
  __shared__ float ltile[LH][LW];
  const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 8;
  stage_planes<CM, T, TW, TH, LH, LW>(tile, ltile, p, x0 - HALO, y0 - HALO);
  __syncthreads();
  const int gx = x0 + threadIdx.x, gy = y0 + threadIdx.y;
  if (gx >= p.W || gy >= p.H) return;
  const int tx = threadIdx.x, ty = threadIdx.y;
  auto lum = [&](int kx, int ky) {
    return CM == kRgb ? ltile[CM == kRgb ? ty + ky : 0][CM == kRgb ? tx + kx : 0] : tile[0][ty + ky][tx + kx];
  };
  float a, b, d;
  structure_tensor<N, true>(lum, p.kp, a, b, d);
  int key = ravu_key(a, b, d, p.kp);
  if (p.keys) p.keys[(size_t)gy * p.W + gx] = key;
  const float4* L = p.lut + (size_t)min(max(key, 0), p.lut_rows - 1) * p.lut_cols;
  float res[C];
#pragma unroll
  for (int c = 0; c < C; c++) res[c] = 0.0f;
#pragma unroll
  for (int q = 0; q < (S / 2 + 3) / 4; q++) {
    const float4 w4 = __ldg(L + q);
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int i = 4 * q + j;
      if (i < S / 2) {
        const float w = j == 0 ? w4.x : (j == 1 ? w4.y : (j == 2 ? w4.z : w4.w));
#pragma unroll
        for (int c = 0; c < C; c++)
          res[c] += (tile[c][ty + i % N][tx + i / N] + tile[c][ty + (S - 1 - i) % N][tx + (S - 1 - i) / N]) * w;
      }
    }
  }
#pragma unroll
  for (int c = 0; c < C; c++) {
    T* o = static_cast<T*>(p.out[c]);
    const size_t op = p.out_pitch[c];
    stp(o + (size_t)(2 * gy) * op + 2 * gx, tile[c][ty + HALO][tx + HALO]);  // input copy
    stp(o + (size_t)(2 * gy + 1) * op + 2 * gx + 1, clampf(res[c], 0.f, 1.f));
  }
}

// Where lattice sample k (grid (k/N, k%N)) of an int10 (L=0) or int01 (L=1)
// pass reads: returns 0 for the input, 1 for int11, with offsets (dx, dy).
// ravu-r3.hook:155-189 (int10) and :289-323 (int01).
template <int N>
__host__ __device__ constexpr int lat_src(int k, int L) {
  return (((k / N + k % N - (N - 1)) % 2 != 0) == (L == 0)) ? 0 : 1;
}
template <int N>
__host__ __device__ constexpr int lat_dx(int k, int L) {
  // s = kx+ky-(N-1); int10: input (s+1)/2, int11 s/2; int01: input s/2, int11 (s-1)/2
  return L == 0 ? (lat_src<N>(k, L) == 0 ? (k / N + k % N - (N - 1) + 1) / 2 : (k / N + k % N - (N - 1)) / 2)
                : (lat_src<N>(k, L) == 0 ? (k / N + k % N - (N - 1)) / 2 : (k / N + k % N - (N - 1) - 1) / 2);
}
template <int N>
__host__ __device__ constexpr int lat_dy(int k, int L) {
  // d = ky-kx; int10: input d/2, int11 (d-1)/2; int01: input (d+1)/2, int11 d/2
  return L == 0 ? (lat_src<N>(k, L) == 0 ? (k % N - k / N) / 2 : (k % N - k / N - 1) / 2)
                : (lat_src<N>(k, L) == 0 ? (k % N - k / N + 1) / 2 : (k % N - k / N) / 2);
}

// int10 + int01 pass (compute/ravu-r3.hook:155-430).
template <int R, int CM, typename T>
__global__ void __launch_bounds__(256) lattice_kernel(const __grid_constant__ RavuArgs p) {
  constexpr int N = 2 * R, S = N * N;
  constexpr int TW = 32 + N - 1, TH = 8 + N - 1;
  constexpr int C = CM == kLuma ? 1 : 3;
  constexpr int LH = CM == kRgb ? TH : 1, LW = CM == kRgb ? TW : 1;
  __shared__ float tin[C][TH][TW];   // input, offsets -(R-1) .. R
  __shared__ float lin[LH][LW];
  __shared__ float t11[C][TH][TW];   // int11, offsets -R .. R-1
  __shared__ float l11[LH][LW];
  const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 8;
  stage_planes<CM, T, TW, TH, LH, LW>(tin, lin, p, x0 - (R - 1), y0 - (R - 1));
  for (int i = threadIdx.y * 32 + threadIdx.x; i < TW * TH; i += 256) {
    int ty = i / TW, tx = i % TW;
    int cx = clampi(x0 - R + tx, 0, p.W - 1), cy = clampi(y0 - R + ty, 0, p.H - 1);
    float v[3];
#pragma unroll
    for (int c = 0; c < C; c++) {
      v[c] = ldp(static_cast<const T*>(p.out[c]) + (size_t)(2 * cy + 1) * p.out_pitch[c] + 2 * cx + 1);
      t11[c][ty][tx] = v[c];
    }
    if (CM == kRgb) l11[CM == kRgb ? ty : 0][CM == kRgb ? tx : 0] = rgb_luma(v[0], v[1], v[2]);
  }
  __syncthreads();
  const int gx = x0 + threadIdx.x, gy = y0 + threadIdx.y;
  if (gx >= p.W || gy >= p.H) return;
  const int tx = threadIdx.x, ty = threadIdx.y;
#pragma unroll
  for (int L = 0; L < 2; L++) {
    auto val = [&](int c, int k) {
      return lat_src<N>(k, L) == 0 ? tin[c][ty + lat_dy<N>(k, L) + R - 1][tx + lat_dx<N>(k, L) + R - 1]
                                   : t11[c][ty + lat_dy<N>(k, L) + R][tx + lat_dx<N>(k, L) + R];
    };
    auto lum = [&](int kx, int ky) {
      const int k = kx * N + ky;
      if (CM != kRgb) return val(0, k);
      return lat_src<N>(k, L) == 0
                 ? lin[CM == kRgb ? ty + lat_dy<N>(k, L) + R - 1 : 0][CM == kRgb ? tx + lat_dx<N>(k, L) + R - 1 : 0]
                 : l11[CM == kRgb ? ty + lat_dy<N>(k, L) + R : 0][CM == kRgb ? tx + lat_dx<N>(k, L) + R : 0];
    };
    float a, b, d;
    structure_tensor<N, true>(lum, p.kp, a, b, d);
    int key = ravu_key(a, b, d, p.kp);
    if (p.keys) p.keys[(size_t)(1 + L) * p.W * p.H + (size_t)gy * p.W + gx] = key;
    const float4* Lr = p.lut + (size_t)min(max(key, 0), p.lut_rows - 1) * p.lut_cols;
    float res[C];
#pragma unroll
    for (int c = 0; c < C; c++) res[c] = 0.0f;
#pragma unroll
    for (int q = 0; q < (S / 2 + 3) / 4; q++) {
      const float4 w4 = __ldg(Lr + q);
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const int i = 4 * q + j;
        if (i < S / 2) {
          const float w = j == 0 ? w4.x : (j == 1 ? w4.y : (j == 2 ? w4.z : w4.w));
#pragma unroll
          for (int c = 0; c < C; c++) res[c] += (val(c, i) + val(c, S - 1 - i)) * w;
        }
      }
    }
#pragma unroll
    for (int c = 0; c < C; c++) {
      T* o = static_cast<T*>(p.out[c]);
      const size_t op = p.out_pitch[c];
      if (L == 0)
        stp(o + (size_t)(2 * gy) * op + 2 * gx + 1, clampf(res[c], 0.f, 1.f));  // int10
      else
        stp(o + (size_t)(2 * gy + 1) * op + 2 * gx, clampf(res[c], 0.f, 1.f));  // int01
    }
  }
}

template <typename T>
int launch_t(const RavuArgs& a, int radius, int cm, cudaStream_t s) {
  dim3 blk(32, 8), grd((a.W + 31) / 32, (a.H + 7) / 8);
#define PZ_LAT(R, CM)                                  \
  do {                                                 \
    int11_kernel<R, CM, T><<<grd, blk, 0, s>>>(a);     \
    lattice_kernel<R, CM, T><<<grd, blk, 0, s>>>(a);   \
  } while (0)
#define PZ_LAT_CM(R)                 \
  if (cm == kLuma) PZ_LAT(R, kLuma); \
  else if (cm == kYuv) PZ_LAT(R, kYuv); \
  else PZ_LAT(R, kRgb)
  if (radius == 2) { PZ_LAT_CM(2); }
  else if (radius == 3) { PZ_LAT_CM(3); }
  else if (radius == 4) { PZ_LAT_CM(4); }
  else return -95;
#undef PZ_LAT_CM
#undef PZ_LAT
  return 0;
}

}  // namespace

int launch_lattice(const RavuArgs& a, int radius, int cm, int dtype, cudaStream_t s) {
  return dtype == 0 ? launch_t<float>(a, radius, cm, s) : launch_t<__half>(a, radius, cm, s);
}

}  // namespace pz
