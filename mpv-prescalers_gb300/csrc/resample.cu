// Resampling around the hook chain: pz_resample.
//
// Two host steps surround a prescaler in mpv and decide what it shows:
//   * a pass's //!OFFSET (ravu-r3.hook:424 "-0.5 -0.5"; nnedi3-nns16-win8x4.hook:95
//     "0 -0.5" and :185 "-0.5 0") announces a pixel shift of its
//     output, which the host folds into its next scaling pass;
//   * a NATIVE hook (compute/ravu-r2-yuv.hook:15) sees the planes merged at
//     luma size, i.e. subsampled chroma already upscaled by --cscale
//     (README.md:50-56).
// Both are one separable interpolation per plane:
//   out(x, y) = sum_i sum_j k(u - i) k(v - j) in(clamp(i), clamp(j)),
//   u = sx * x + ox,  v = sy * y + oy,
// with texel centres at integer coordinates and clamp-to-edge borders.
// k is the bilinear tent or the Catmull-Rom cubic (Keys' cubic convolution
// kernel with a = -1/2).  One thread per output texel; the 2x2 or 4x4 input
// footprint comes through L1 (a variant staging each block's footprint in
// shared memory first measured 10 % slower).
#include "../../include/prescale.h"
#include "kernels.h"
#include "model.h"

namespace pz {
namespace {

struct ResampleArgs {
  const void* in;
  void* out;
  int in_w, in_h, in_pitch;
  int out_w, out_h, out_pitch;
  float sx, ox, sy, oy;
};

// Catmull-Rom weights of the 4 taps floor(u)-1 .. floor(u)+2 at fraction t.
__device__ __forceinline__ void cubic_weights(float t, float (&w)[4]) {
  const float t2 = t * t, t3 = t2 * t;
  w[0] = 0.5f * (-t3 + 2.0f * t2 - t);
  w[1] = 0.5f * (3.0f * t3 - 5.0f * t2 + 2.0f);
  w[2] = 0.5f * (-3.0f * t3 + 4.0f * t2 + t);
  w[3] = 0.5f * (t3 - t2);
}

template <int TAPS, typename T>
__global__ void __launch_bounds__(256) resample_kernel(const ResampleArgs a) {
  const int x = blockIdx.x * 32 + (threadIdx.x & 31);
  const int y = blockIdx.y * 8 + (threadIdx.x >> 5);
  if (x >= a.out_w || y >= a.out_h) return;
  const T* in = static_cast<const T*>(a.in);
  const float u = fmaf(a.sx, (float)x, a.ox), v = fmaf(a.sy, (float)y, a.oy);
  const float fu = floorf(u), fv = floorf(v);
  const int iu = (int)fu, iv = (int)fv;
  float wx[4], wy[4];
  if (TAPS == 2) {
    wx[0] = 1.0f - (u - fu);
    wx[1] = u - fu;
    wy[0] = 1.0f - (v - fv);
    wy[1] = v - fv;
  } else {
    cubic_weights(u - fu, wx);
    cubic_weights(v - fv, wy);
  }
  constexpr int K0 = TAPS == 2 ? 0 : -1;
  int cx[TAPS];
#pragma unroll
  for (int i = 0; i < TAPS; i++) cx[i] = clampi(iu + K0 + i, 0, a.in_w - 1);
  float acc = 0.0f;
#pragma unroll
  for (int j = 0; j < TAPS; j++) {
    const T* row = in + (size_t)clampi(iv + K0 + j, 0, a.in_h - 1) * a.in_pitch;
    float r = 0.0f;
#pragma unroll
    for (int i = 0; i < TAPS; i++) r += wx[i] * ldp(row + cx[i]);
    acc += wy[j] * r;
  }
  stp(static_cast<T*>(a.out) + (size_t)y * a.out_pitch + x, acc);
}

int check_rs_plane(const pz_plane* p, const char* what) {
  if (!p || !p->data) return set_error(PZ_EINVAL, "%s: null plane", what);
  if (p->width <= 0 || p->height <= 0 || p->pitch < p->width)
    return set_error(PZ_EINVAL, "%s: bad size %dx%d pitch %d", what, p->width, p->height, p->pitch);
  if (p->dtype != PZ_F32 && p->dtype != PZ_F16) return set_error(PZ_EINVAL, "%s: unknown dtype %d", what, p->dtype);
  if (reinterpret_cast<uintptr_t>(p->data) % (p->dtype == PZ_F32 ? 4 : 2))
    return set_error(PZ_EINVAL, "%s: misaligned base", what);
  return PZ_OK;
}

}  // namespace
}  // namespace pz

extern "C" int pz_resample(const pz_plane* in, pz_plane* out, float sx, float ox, float sy, float oy, int filter,
                           void* stream) {
  int rc;
  if ((rc = pz::check_rs_plane(in, "in")) || (rc = pz::check_rs_plane(out, "out"))) return rc;
  if (in->dtype != out->dtype) return pz::set_error(PZ_EINVAL, "input and output dtypes differ");
  if (filter != PZ_FILTER_BILINEAR && filter != PZ_FILTER_CATMULL_ROM)
    return pz::set_error(PZ_EINVAL, "unknown filter %d", filter);
  // every sample position must stay a finite float well inside int range
  const float lim = 1.0e7f;
  const float ux0 = ox, ux1 = sx * (float)(out->width - 1) + ox;
  const float vy0 = oy, vy1 = sy * (float)(out->height - 1) + oy;
  if (!(fabsf(ux0) < lim && fabsf(ux1) < lim && fabsf(vy0) < lim && fabsf(vy1) < lim))
    return pz::set_error(PZ_EINVAL, "sample positions out of range");
  pz::ResampleArgs a{in->data, out->data, in->width, in->height, in->pitch,
                     out->width, out->height, out->pitch, sx, ox, sy, oy};
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const dim3 grid((out->width + 31) / 32, (out->height + 7) / 8);
  const bool f16 = in->dtype == PZ_F16;
  if (filter == PZ_FILTER_BILINEAR) {
    if (f16) pz::resample_kernel<2, __half><<<grid, 256, 0, s>>>(a);
    else pz::resample_kernel<2, float><<<grid, 256, 0, s>>>(a);
  } else {
    if (f16) pz::resample_kernel<4, __half><<<grid, 256, 0, s>>>(a);
    else pz::resample_kernel<4, float><<<grid, 256, 0, s>>>(a);
  }
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return pz::set_error(PZ_EIO, "resample launch: %s", cudaGetErrorString(e));
  return PZ_OK;
}
