// NNEDI3 doubling pass, plain FP32 on the CUDA cores.
//
// Reference: nnedi3-nns16-win8x4.hook:15-104 (double_y: 8x4 window,
// normalisation, nns neuron pairs, softmax-weighted Elliott blend) and its
// transposed twin double_x (:120-200); compute/nnedi3-nns128-win8x6.hook:
// 15-232 fuses each double pass with its combine (both pixels written).
//
// One thread per interpolated pixel; the window tile sits in shared memory,
// the weights of every neuron (both branches, FP32, [nns][2][T]) too, read
// as warp-uniform float4 broadcasts.  The window is centred before the dot
// products: <x, A> = <x - mean, A> + mean * sum(A), with sum(A) precomputed
// in double on the host, which keeps FP32 cancellation out of the
// pre-activations.  The variance is taken two-pass, sum((x - mean)^2) / T.
#include "kernels.h"

namespace pz {
namespace {

template <int WH, bool XP, typename T>
__global__ void __launch_bounds__(256) nn_simt_kernel(const __grid_constant__ NnArgs p) {
  constexpr int NT = 8 * WH;
  constexpr int DY0 = -(WH / 2 - 1);
  constexpr int OX0 = XP ? DY0 : -3, OX1 = XP ? WH / 2 : 4;
  constexpr int OY0 = XP ? -3 : DY0, OY1 = XP ? 4 : WH / 2;
  constexpr int TW = 32 + OX1 - OX0, TH = 8 + OY1 - OY0;
  __shared__ float tile[TH][TW];
  extern __shared__ float4 wsm[];  // [nns][2][NT/4] weights, then [nns][4] (csA, csB, bA, bB)
  const int nns = p.nns;
  const float4* gw = reinterpret_cast<const float4*>(p.wts);
  const int nw4 = nns * 2 * NT / 4;
  for (int i = threadIdx.y * 32 + threadIdx.x; i < nw4; i += 256) wsm[i] = __ldg(gw + i);
  float4* aux = wsm + nw4;
  for (int k = threadIdx.y * 32 + threadIdx.x; k < nns; k += 256)
    aux[k] = make_float4(__ldg(p.cs + 2 * k), __ldg(p.cs + 2 * k + 1), __ldg(p.bias + 2 * k), __ldg(p.bias + 2 * k + 1));
  const T* in = static_cast<const T*>(p.in);
  const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 8;
  for (int i = threadIdx.y * 32 + threadIdx.x; i < TW * TH; i += 256) {
    int ty = i / TW, tx = i % TW;
    int gx = clampi(x0 + OX0 + tx, 0, p.W - 1), gy = clampi(y0 + OY0 + ty, 0, p.H - 1);
    tile[ty][tx] = ldp(in + (size_t)gy * p.in_pitch + gx);
  }
  __syncthreads();
  const int gx = x0 + threadIdx.x, gy = y0 + threadIdx.y;
  if (gx >= p.W || gy >= p.H) return;
  float xv[NT];
  float sum = 0.0f;
#pragma unroll
  for (int t = 0; t < NT; t++) {
    const int dx = t % 8 - 3, dy = t / 8 + DY0;
    const int ox = XP ? dy : dx, oy = XP ? dx : dy;
    xv[t] = tile[(int)threadIdx.y + oy - OY0][(int)threadIdx.x + ox - OX0];
    sum += xv[t];
  }
  const float mean = sum / (float)NT;
  float var = 0.0f;
#pragma unroll
  for (int t = 0; t < NT; t++) {
    xv[t] -= mean;
    var += xv[t] * xv[t];
  }
  var /= (float)NT;
  // mstd2 = var >= eps ? inversesqrt(var) : 0; mstd1 = var * mstd2
  const float invstd = var >= kFltEps ? 1.0f / sqrtf(var) : 0.0f;
  const float stdv = var * invstd;
  float wsum = 0.0f, vsum = 0.0f;
  for (int k = 0; k < nns; k++) {
    const float4* wa = wsm + k * (NT / 2);
    float s1 = 0.0f, s2 = 0.0f;
#pragma unroll
    for (int q = 0; q < NT / 4; q++) {
      const float4 w = wa[q];
      s1 += xv[4 * q] * w.x + xv[4 * q + 1] * w.y + xv[4 * q + 2] * w.z + xv[4 * q + 3] * w.w;
    }
#pragma unroll
    for (int q = 0; q < NT / 4; q++) {
      const float4 w = wa[NT / 4 + q];
      s2 += xv[4 * q] * w.x + xv[4 * q + 1] * w.y + xv[4 * q + 2] * w.z + xv[4 * q + 3] * w.w;
    }
    const float4 c = aux[k];
    s1 = (s1 + mean * c.x) * invstd + c.z;
    s2 = (s2 + mean * c.y) * invstd + c.w;
    const float e = expf(s1);
    wsum += e;
    vsum += e * (s2 / (1.0f + fabsf(s2)));
  }
  const float v = clampf(mean + 5.0f * vsum / wsum * stdv, 0.0f, 1.0f);
  T* out = static_cast<T*>(p.out);
  const float orig = tile[(int)threadIdx.y - OY0][(int)threadIdx.x - OX0];
  if (XP) {
    stp2(out + (size_t)gy * p.out_pitch + 2 * gx, orig, v);
  } else {
    stp(out + (size_t)(2 * gy) * p.out_pitch + gx, orig);
    stp(out + (size_t)(2 * gy + 1) * p.out_pitch + gx, v);
  }
}

template <int WH, bool XP, typename T>
int launch_one(const NnArgs& a, cudaStream_t s) {
  const size_t smem = ((size_t)a.nns * 2 * 8 * WH + (size_t)a.nns * 4) * sizeof(float);
  auto kern = nn_simt_kernel<WH, XP, T>;
  static size_t configured[64] = {};  // largest dynamic smem enabled, per device
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return -95;
  if (smem > 48 * 1024 && smem > configured[dev]) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return -5;
    configured[dev] = smem;
  }
  dim3 blk(32, 8), grd((a.W + 31) / 32, (a.H + 7) / 8);
  kern<<<grd, blk, smem, s>>>(a);
  return 0;
}

template <typename T>
int launch_t(const NnArgs& a, bool xp, cudaStream_t s) {
  if (a.win_h == 4) return xp ? launch_one<4, true, T>(a, s) : launch_one<4, false, T>(a, s);
  if (a.win_h == 6) return xp ? launch_one<6, true, T>(a, s) : launch_one<6, false, T>(a, s);
  return -95;
}

}  // namespace

int launch_nnedi3_simt(const NnArgs& a, bool xpass, int dtype, cudaStream_t s) {
  return dtype == 0 ? launch_t<float>(a, xpass, s) : launch_t<__half>(a, xpass, s);
}

}  // namespace pz
