// Shared device code for the prescaler kernels (sm_103a).
//
// The arithmetic mirrors the reference shaders expression by expression
// where that matters for the key (the quantised LUT row):
//   structure tensor   ravu-lite-r3.hook:48-76, ravu-r3.hook:58-107
//   eigen/key          ravu-lite-r3.hook:77-88, ravu-r3.hook:108-125
// All key math is FP32; see ravu_key for how each threshold test is evaluated.
#pragma once
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace pz {

constexpr float kFltEps = 1.192092896e-7f;   // the shaders' epsilon literal
constexpr float kPi = 3.141592653589793f;    // the shaders' pi literal

// Key quantisation constants of one model (kernel parameter).
struct KeyParams {
  float gw[36];      // Gaussian weights of the gradient points (geometry order)
  float gwf[36];     // gw * c^2 where both stencils of a point have the same scale c
                     // (1 one-sided, 1/2 central, 1/12 four-tap), else gw
  float thr[3];      // strength thresholds (lite, zoom: 3; 3x: 2)
  int n_thr;
  int log2_mode;     // ravu: strength = clamp(floor(log2(l*scale+eps)), 0, max)
  float log2_scale;
  float log2_max;
  float coh0, coh1;  // coherence thresholds
  int n_strength;    // strength levels
  int rows;          // LUT keys (24 * n_strength * 3)
};

// Device-side error word shared by all kernels: first failure wins.
enum : int { kErrNone = 0, kErrTileOverflow = 1, kErrWaitTimeout = 2, kErrQueue = 3 };

// ------------------------------------------------------------- plane I/O --
__device__ __forceinline__ float ldp(const float* p) { return __ldg(p); }
__device__ __forceinline__ float ldp(const __half* p) {
  return __half2float(__ushort_as_half(__ldg(reinterpret_cast<const unsigned short*>(p))));
}
__device__ __forceinline__ void stp(float* p, float v) { *p = v; }
__device__ __forceinline__ void stp(__half* p, float v) { *p = __float2half_rn(v); }
// two horizontally adjacent pixels (p must be 2-element aligned)
__device__ __forceinline__ void stp2(float* p, float a, float b) {
  *reinterpret_cast<float2*>(p) = make_float2(a, b);
}
__device__ __forceinline__ void stp2(__half* p, float a, float b) {
  *reinterpret_cast<__half2*>(p) = __floats2half2_rn(a, b);
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
__device__ __forceinline__ float clampf(float v, float lo, float hi) { return fminf(fmaxf(v, lo), hi); }
// GLSL mod(): x - y * floor(x / y)
__device__ __forceinline__ float gl_mod(float x, float y) { return x - y * floorf(x / y); }

// --------------------------------------------------- structure tensor -----
// Gradient stencil at grid position p along one axis of an N-tap window:
// one-sided at the border, central /2 inside, and (FOUR: ravu, ravu-zoom)
// (-s[p+2] + 8 s[p+1] - 8 s[p-1] + s[p-2]) / 12 where both exist.
// stencil_kind: 0 one-sided, 1 central, 2 four-tap (also used on the host
// to scale the weights of KeyParams::gwf).
__host__ __device__ constexpr int stencil_kind(int n, bool four, int p) {
  return (p == 0 || p == n - 1) ? 0 : ((four && p >= 2 && p <= n - 3) ? 2 : 1);
}

// The stencil without its scale (1, 1/2, 1/12).
template <int N, bool FOUR, class G>
__device__ __forceinline__ float deriv_unscaled(const G& s, int p) {
  if (p == 0) return s(1) - s(0);
  if (p == N - 1) return s(N - 1) - s(N - 2);
  if (FOUR && p >= 2 && p <= N - 3) return -s(p + 2) + 8.0f * s(p + 1) - 8.0f * s(p - 1) + s(p - 2);
  return s(p + 1) - s(p - 1);
}

template <int N, bool FOUR, class G>
__device__ __forceinline__ float deriv(const G& s, int p) {
  if (p == 0) return s(1) - s(0);
  if (p == N - 1) return s(N - 1) - s(N - 2);
  if (FOUR && p >= 2 && p <= N - 3)
    return (-s(p + 2) + 8.0f * s(p + 1) - 8.0f * s(p - 1) + s(p - 2)) * (1.0f / 12.0f);
  return (s(p + 1) - s(p - 1)) * 0.5f;
}

// Gaussian-weighted sum of (gx^2, gx gy, gy^2) over the gradient points:
// the whole window when N <= 4, else the window minus a one-tap border.
// `get(kx, ky)` returns the key input at window grid (kx, ky).  PACKED: a
// and d accumulate as one FP32x2 pair, a += gx (gx w), d += gy (gy w),
// b += (gx w) gy (three instructions per point instead of six), and where
// both stencils of a point share one scale c the scale moves into the weight
// (gwf = gw c^2: the unscaled differences are used).  Each term then rounds
// a few times differently from the shader's gx * gx * w, far inside the
// key's FP32 boundary budget.
template <int N, bool FOUR, bool PACKED = true, class Get>
__device__ __forceinline__ void structure_tensor(const Get& get, const KeyParams& kp, float& a,
                                                 float& b, float& d) {
  constexpr int P0 = N <= 4 ? 0 : 1;
  constexpr int P1 = N <= 4 ? N : N - 1;
  float2 ad = make_float2(0.0f, 0.0f);
  a = 0.0f;
  b = 0.0f;
  d = 0.0f;
  int i = 0;
#pragma unroll
  for (int px = P0; px < P1; px++) {
#pragma unroll
    for (int py = P0; py < P1; py++) {
      const bool fold = PACKED && stencil_kind(N, FOUR, px) == stencil_kind(N, FOUR, py);
      auto sx = [&](int q) { return get(q, py); };
      auto sy = [&](int q) { return get(px, q); };
      const float gx = fold ? deriv_unscaled<N, FOUR>(sx, px) : deriv<N, FOUR>(sx, px);
      const float gy = fold ? deriv_unscaled<N, FOUR>(sy, py) : deriv<N, FOUR>(sy, py);
      const float w = fold ? kp.gwf[i] : kp.gw[i];
      i++;
      if constexpr (PACKED) {
        const float2 g2 = make_float2(gx, gy);
        const float2 gw2 = __fmul2_rn(g2, make_float2(w, w));
        ad = __ffma2_rn(g2, gw2, ad);
        b = fmaf(gw2.x, gy, b);
      } else {
        a += gx * gx * w;
        b += gx * gy * w;
        d += gy * gy * w;
      }
    }
  }
  if constexpr (PACKED) {
    a = ad.x;
    d = ad.y;
  }
}

__device__ __forceinline__ float sqrt_approx(float x) {
  float r;
  asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));  // NaN for x < 0, as in GLSL
  return r;
}

// floor(24 * theta / pi) with theta = mod(atan(y, x) + pi, pi) in [0, pi),
// without the arctangent: the direction is folded into [0, pi/4] (a turn by
// -pi/2, then a mirror about the diagonal) and the sector boundaries
// k*pi/24 below it are counted by comparing y with tan(k*pi/24) * x.  Only
// directions within FP32 rounding of a boundary can land in the neighbouring
// sector (the oracle's boundary keys); a NaN component gives sector 0.
__device__ __forceinline__ float angle_sector(float x, float y) {
  if (y < 0.0f || (y == 0.0f && x < 0.0f)) {  // theta + pi: same direction mod pi
    x = -x;
    y = -y;
  }
  float base = 0.0f;
  if (x < 0.0f) {  // theta in (pi/2, pi): turn by -pi/2
    const float t = x;
    x = y;
    y = -t;
    base = 12.0f;
  }
  const bool mirror = y > x;  // above pi/4: theta'' = pi/2 - theta'
  if (mirror) {
    const float t = x;
    x = y;
    y = t;
  }
  const float s = (float)((int)(y >= 0.131652498f * x) + (int)(y >= 0.267949192f * x) +
                          (int)(y >= 0.414213562f * x) + (int)(y >= 0.577350269f * x) +
                          (int)(y >= 0.767326988f * x) + (int)(y >= x));
  return base + (mirror ? 11.0f - s : s);
}

// Eigen analysis + quantisation -> raw key (not clamped to the LUT).
// ravu-lite-r3.hook:77-88 (strength thresholds), ravu-r3.hook:121-125 (log2).
//
// The quantised outputs equal the shader's; only the way each threshold test
// is evaluated changes, so results can differ only where a quantity lies
// within FP32 rounding of a threshold (the oracle's boundary keys):
//   * angle: the sector by comparisons with tan(k*pi/24) (angle_sector)
//     instead of floor(atan(.) * 24 / pi);
//   * coherence: mu >= c  <=>  (sqrtL1 - sqrtL2) >= c * (sqrtL1 + sqrtL2),
//     no division; NaN (L2 < 0) still fails every test -> 0, and the
//     sqrtL1 + sqrtL2 < eps gate still forces 0;
//   * log2 strength: floor(log2(v)) is the unbiased exponent of v (> 0).
__device__ __forceinline__ int ravu_key(float a, float b, float d, const KeyParams& kp) {
  float T = a + d, D = a * d - b * b;
  float delta = sqrt_approx(fmaxf(T * T * 0.25f - D, 0.0f));
  float L1 = T * 0.5f + delta, L2 = T * 0.5f - delta;
  float sqrtL1 = sqrt_approx(L1), sqrtL2 = sqrt_approx(L2);
  const float angle = fabsf(b) < kFltEps ? 0.0f : angle_sector(b, L1 - a);
  float lambda = sqrtL1;
  float strength;
  if (kp.log2_mode) {
    const float v = lambda * kp.log2_scale + kFltEps;
    strength = clampf((float)((__float_as_int(v) >> 23) - 127), 0.0f, kp.log2_max);
  } else if (kp.n_thr == 3) {
    strength = lambda >= kp.thr[1] ? (lambda >= kp.thr[2] ? 3.0f : 2.0f) : (lambda >= kp.thr[0] ? 1.0f : 0.0f);
  } else {
    strength = lambda >= kp.thr[1] ? 2.0f : (lambda >= kp.thr[0] ? 1.0f : 0.0f);
  }
  const float ssum = sqrtL1 + sqrtL2, sdif = sqrtL1 - sqrtL2;
  float coherence = 0.0f;
  if (!(ssum < kFltEps)) coherence = sdif >= kp.coh1 * ssum ? 2.0f : (sdif >= kp.coh0 * ssum ? 1.0f : 0.0f);
  return (int)((angle * (float)kp.n_strength + strength) * 3.0f + coherence);
}

// Anti-ringing powers of one value as FP32x2 pairs: (h^32, l^32) and
// (h^33, l^33) with h = 0.1 + v, l = 1.1 - v, pow(x, 32) by five squarings
// (ravu-lite-ar-r3.hook:91-98); each lane rounds as a scalar FMUL would.
__device__ __forceinline__ void ar_pow2(float v, float2& p32, float2& p33) {
  const float2 hl = __ffma2_rn(make_float2(v, v), make_float2(1.0f, -1.0f), make_float2(0.1f, 1.1f));
  float2 q = hl;
#pragma unroll
  for (int i = 0; i < 5; i++) q = __fmul2_rn(q, q);
  p32 = q;
  p33 = __fmul2_rn(q, hl);
}

// lo = 1.1 - lo2/lo; hi = hi2/hi - 0.1; mix(res, clamp(res, lo, hi), s).
// The quotients are approximate (__fdividef, about 2 ulp, the precision a
// shader's division has): they only move the clamp bounds, by < 3e-7.  Both
// operands are scaled by 2^24 first, so that a subnormal denominator
// (positive weights summing below ~1e-6) still has a finite reciprocal; for
// every other denominator the scaling changes no bit of the quotient.
__device__ __forceinline__ float ar_quot(float n, float d) {
  return __fdividef(n * 16777216.0f, d * 16777216.0f);
}
__device__ __forceinline__ float ar_finish(float res, float lo, float hi, float lo2, float hi2, float s) {
  float lob = 1.1f - ar_quot(lo2, lo);
  float hib = ar_quot(hi2, hi) - 0.1f;
  float c = fminf(fmaxf(res, lob), hib);
  return res * (1.0f - s) + c * s;
}

// Rec.709 luma of an RGB sample (ravu-r2-rgb.hook:21 color_primary).
__device__ __forceinline__ float rgb_luma(float r, float g, float b) {
  return r * 0.2126f + g * 0.7152f + b * 0.0722f;
}

}  // namespace pz
