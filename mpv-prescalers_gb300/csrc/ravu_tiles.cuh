// RAVU tile programs: one CTA of 32 x TR threads computes one tile of outputs.
//
// Each program is a struct with the shared-memory bytes it needs and a
// device `run(p, x0, y0, smem)` that stages the tile (plus its radius halo)
// and computes it.  The per-model kernels (ravu_lite.cu, ravu_lattice.cu,
// ravu_zoom.cu) launch one CTA per tile; the persistent batch kernel
// (batch.cu) feeds many programs of many frames to the same CTAs.
//
// References (per program):
//   LiteTile    compute/ravu-lite-ar-r3.hook:15-171, ravu-lite-r3.hook:15-131
//   ThreeXTile  compute/ravu-3x-r2.hook:15-115
//   Int11Tile   ravu-r3.hook:15-146 (compute/ravu-r3.hook:15-154)
//   LatticeTile ravu-r3.hook:148-437 (compute/ravu-r3.hook:155-430)
//   ZoomTile    ravu-zoom-r2.hook:15-139, compute/ravu-zoom-ar-r2-rgb.hook:15-238
//
// Input tiles are 32 x TR input pixels (zoom: output pixels), TR = 4, 8 or 16
// rows (a template argument of every program; 8 is the reference's own
// workgroup height, compute/ravu-lite-r3.hook:22); thread t handles column
// t % 32 of row t / 32.  Out-of-range reads replicate the edge texel (the mpv
// texture border mode).
#pragma once
#include <cstddef>
#include <cstring>

#include "async.cuh"
#include "kernels.h"

namespace pz {

// Tile width in pixels (one warp per tile row); persistent batches run tiles
// of kBatchTileRows rows.
constexpr int kTileW = 32, kBatchTileRows = 8;

__host__ __device__ constexpr int cabs(int v) { return v < 0 ? -v : v; }

// Stage all planes of a frame; RGB also gets a Rec.709 luma tile (the key
// input); luma and yuv take their key input from plane 0.
// NT threads share the work.
template <int CM, int TW, int TH, int NT, typename T>
__device__ __forceinline__ void stage_planes(float* tile, float* ltile, const RavuArgs& p, int x0, int y0) {
  constexpr int C = CM == kLuma ? 1 : 3;
  for (int i = threadIdx.x; i < TW * TH; i += NT) {
    const int ty = i / TW, tx = i % TW;
    const int gx = clampi(x0 + tx, 0, p.W - 1), gy = clampi(y0 + ty, 0, p.H - 1);
    float v[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int c = 0; c < C; c++) {
      v[c] = ldp(static_cast<const T*>(p.in[c]) + (size_t)gy * p.in_pitch[c] + gx);
      tile[c * TW * TH + i] = v[c];
    }
    if (CM == kRgb) ltile[i] = rgb_luma(v[0], v[1], v[2]);
  }
}

// ---------------------------------------------------------- TMA staging ---
// Interior tiles (window fully inside the plane) can be staged by TMA: one
// 2-D box per plane lands in shared memory, then one pass converts it to the
// float tile the programs read.  Border tiles keep the clamped loads above,
// because TMA fills out-of-range texels with zeros, not the edge value.  The
// box starts at the tile origin rounded down to 8 columns, so its x
// coordinate is 16-byte aligned for FP32 and FP16 planes.
struct TmaMaps {
  CUtensorMap map[3];
};

struct TmaCtx {
  const CUtensorMap* map;  // one per plane (kernel parameter or global memory); null: clamped loads
  uint32_t mbar;           // shared mbarrier (count 1)
  unsigned char* raw;      // landing area, 128-byte aligned
  uint32_t phase;          // parity of the mbarrier's next completion (flips per TMA-staged tile)
  int dead;                // a wait timed out: this CTA stages by clamped loads from now on
};

template <int TW>
__host__ __device__ constexpr int tma_box_w() {
  return (TW + 7 + 7) & ~7;  // up to 7 lead columns from rounding the start down
}
template <int TW, int TH, typename T>
__host__ __device__ constexpr uint32_t tma_plane_bytes() {
  return ((uint32_t)tma_box_w<TW>() * TH * sizeof(T) + 127u) & ~127u;
}

__device__ __forceinline__ float lds_f(const float* p) { return *p; }
__device__ __forceinline__ float lds_f(const __half* p) { return __half2float(*p); }

// Stage a w x h window whose first texel is column `off` of a bw x bh TMA
// box at (bx, by) (bx a multiple of 8): thread 0 issues one box per plane
// into the landing area (plane stride pb bytes), the CTA waits for it, and
// the window is converted to the float tile (row pitch dp, plane stride
// dps; RGB also the luma tile).  Returns 1, or -1 when the copy did not
// complete within the wait bound (error word set, the tile abandoned and TMA
// off for the rest of the CTA).  The outcome of the wait is made uniform across the
// CTA, so every thread takes the same path through the tile's barriers.
template <int CM, int NT, typename T>
__device__ __forceinline__ int tma_stage_box(const RavuArgs& p, TmaCtx* t, int bx, int by, int bw, int bh,
                                             uint32_t pb, int off, int w, int h, int dp, int dps, float* tile,
                                             float* ltile) {
  constexpr int C = CM == kLuma ? 1 : 3;
  if (threadIdx.x == 0) {
    mbar_arrive_expect_tx(t->mbar, (uint32_t)C * bw * bh * sizeof(T));
#pragma unroll
    for (int c = 0; c < C; c++) tma_load_2d(t->raw + c * pb, &t->map[c], bx, by, t->mbar);
  }
  if (!__syncthreads_and(mbar_wait_bounded(t->mbar, t->phase))) {
    if (threadIdx.x == 0 && p.err) atomicCAS(p.err, 0, kErrWaitTimeout);
    t->dead = 1;
    return -1;
  }
  t->phase ^= 1u;
  for (int i = threadIdx.x; i < w * h; i += NT) {
    const int ty = i / w, tx = i % w;
    float v[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int c = 0; c < C; c++) {
      v[c] = lds_f(reinterpret_cast<const T*>(t->raw + c * pb) + ty * bw + tx + off);
      tile[c * dps + ty * dp + tx] = v[c];
    }
    if (CM == kRgb) ltile[ty * dp + tx] = rgb_luma(v[0], v[1], v[2]);
  }
  return 1;
}

// The TW x TH frame tile at (x0, y0) by TMA: 1 staged; 0 not an interior
// tile, or no maps (use clamped loads); -1 the wait timed out.
template <int CM, int TW, int TH, int NT, typename T>
__device__ int stage_planes_tma(const RavuArgs& p, TmaCtx* t, int x0, int y0, float* tile, float* ltile) {
  if (!t || !t->map || t->dead || x0 < 0 || y0 < 0 || x0 + TW > p.W || y0 + TH > p.H) return 0;
  const int bx = x0 & ~7;
  return tma_stage_box<CM, NT, T>(p, t, bx, y0, tma_box_w<TW>(), TH, tma_plane_bytes<TW, TH, T>(), x0 - bx, TW, TH,
                                  TW, TW * TH, tile, ltile);
}

// A CTA whose TMA wait timed out may still have that copy in flight into its
// landing area: before the CTA exits, thread 0 waits (bounded again) for the
// outstanding phase, so the copy never lands in shared memory that another
// CTA owns.  Nothing else touches the landing area or the mbarrier once the
// CTA is marked dead.
__device__ __forceinline__ void tma_drain(const TmaCtx* t) {
  if (t && t->dead && threadIdx.x == 0) (void)mbar_wait_bounded(t->mbar, t->phase);
}

// Stage the frame tile by TMA when possible, else by clamped loads.
// Returns false only when a TMA wait timed out (the tile is abandoned).
template <int CM, int TW, int TH, int NT, typename T>
__device__ __forceinline__ bool stage_frame(const RavuArgs& p, TmaCtx* t, int x0, int y0, float* tile,
                                            float* ltile) {
  const int r = stage_planes_tma<CM, TW, TH, NT, T>(p, t, x0, y0, tile, ltile);
  if (r == 0) stage_planes<CM, TW, TH, NT, T>(tile, ltile, p, x0, y0);
  return r >= 0;
}


// One LUT texel: FP32 (float4) or, in the fast form, FP16 (4 halves in a
// uint2, half the L1 traffic of the per-pixel row gathers).
template <bool H16>
__device__ __forceinline__ float4 lut_texel(const float4* f, const uint2* h, size_t i) {
  if constexpr (H16) {
    const uint2 q = __ldg(h + i);
    const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&q.x));
    const float2 b = __half22float2(*reinterpret_cast<const __half2*>(&q.y));
    return make_float4(a.x, a.y, b.x, b.y);
  } else {
    return __ldg(f + i);
  }
}

// Two adjacent FP32 texels i, i+1 (i even, row pitch even) as one 32-byte load.
__device__ __forceinline__ void lut_pair_f32(const float4* f, size_t i, float4& a, float4& b) {
  asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
      : "l"(f + i));
}

// Two adjacent FP16 texels i, i+1 (i even) as one 16-byte load.
__device__ __forceinline__ void lut_pair_h16(const uint2* h, size_t i, float4& a, float4& b) {
  const uint4 q = __ldg(reinterpret_cast<const uint4*>(h + i));
  const float2 a01 = __half22float2(*reinterpret_cast<const __half2*>(&q.x));
  const float2 a23 = __half22float2(*reinterpret_cast<const __half2*>(&q.y));
  const float2 b01 = __half22float2(*reinterpret_cast<const __half2*>(&q.z));
  const float2 b23 = __half22float2(*reinterpret_cast<const __half2*>(&q.w));
  a = make_float4(a01.x, a01.y, a23.x, a23.y);
  b = make_float4(b01.x, b01.y, b23.x, b23.y);
}

// ------------------------------------------------------------ ravu-lite ---
// Does lite LUT column c take part in the anti-ringing sums?  r2: every
// tap; r3/r4: the 13-tap diamond |dx|+|dy| <= 2 (ravu-lite-ar-r3.hook:93-170).
template <int R>
__host__ __device__ constexpr bool lite_ar_col(int c) {
  return R == 2 || cabs(c / (2 * R - 1) - (R - 1)) + cabs(c % (2 * R - 1) - (R - 1)) <= 2;
}

template <int R, bool AR, typename T, bool H16 = false, int TR = 8>
struct LiteTile {
  static constexpr int N = 2 * R - 1, S = N * N, HALO = R - 1;
  static constexpr int kRows = TR, kThreads = kTileW * TR;
  static constexpr bool kOutputTiles = false;
  static constexpr int TW = kTileW + N - 1, TH = TR + N - 1;
  // the value tile; the anti-ringing powers are formed per tap in registers
  // (ar_pow2): a shared table of each texel's four powers, formed once per
  // texel, measured 2-13 % slower (an extra barrier, 8 KB more shared memory
  // per CTA and a 16-byte shared load per tap)
  static constexpr size_t smem_bytes = (size_t)((TW * TH + 3) & ~3) * 4;

  static constexpr int kPlanes = 1;
  // ravu-lite-ar-r4 at <= 48 registers (5 CTAs of 8 rows per SM) measured
  // 2 % faster; the other radii lose more to spills than they gain
  static constexpr int kMaxRegs = (R == 4 && AR) ? 48 : 0;
  // ravu-lite-ar-r2 / -r3 measured 2-5 % slower with the packed structure
  // tensor (register allocation of the anti-ringing sums)
  static constexpr bool kPackedTensor = !(R <= 3 && AR);
  using Elem = T;

  __device__ static void run(const RavuArgs& p, int x0, int y0, float* smem, TmaCtx* tma = nullptr) {
    float* tile = smem;
    if (!stage_frame<kLuma, TW, TH, kThreads, T>(p, tma, x0 - HALO, y0 - HALO, tile, nullptr)) return;
    __syncthreads();
    const int tx = threadIdx.x % kTileW, ty = threadIdx.x / kTileW;
    const int gx = x0 + tx, gy = y0 + ty;
    if (gx >= p.W || gy >= p.H) return;
    auto get = [&](int kx, int ky) { return tile[(ty + ky) * TW + tx + kx]; };
    float a, b, d;
    structure_tensor<N, false, kPackedTensor>(get, p.kp, a, b, d);
    const int key = ravu_key(a, b, d, p.kp);
    if (p.keys) p.keys[(size_t)gy * p.W + gx] = key;
    const size_t row = (size_t)min(max(key, 0), p.lut_rows - 1) * (H16 ? p.lut_h_pitch : p.lut_cols);
    float4 w_next;  // H16: the odd texel of the pair loaded at the even one
    static_assert(S / 2 % 2 == 0, "texel pairs start at even columns");
    // FP32x2 sums: P = sum va*w, Q = sum vb*w, res = P + Q.wzyx; the
    // anti-ringing sums of output k as (hi, lo) and (hi2, lo2) pairs
    float2 P01 = make_float2(0.f, 0.f), P23 = P01, Q01 = P01, Q23 = P01;
    float2 HL[4], HL3[4];
#pragma unroll
    for (int k = 0; k < 4; k++) HL[k] = HL3[k] = P01;
#pragma unroll
    for (int c = 0; c < S / 2; c++) {
      float4 w;
      if constexpr (H16) {
        if (c % 2 == 0) lut_pair_h16(p.lut_h, row + c, w, w_next);
        else w = w_next;
      } else {
        w = __ldg(p.lut + row + c);
      }
      const float va = get(c / N, c % N), vb = get((S - 1 - c) / N, (S - 1 - c) % N);
      const float2 w01 = make_float2(w.x, w.y), w23 = make_float2(w.z, w.w);
      const float2 a2 = make_float2(va, va), b2 = make_float2(vb, vb);
      P01 = __ffma2_rn(a2, w01, P01);
      P23 = __ffma2_rn(a2, w23, P23);
      Q01 = __ffma2_rn(b2, w01, Q01);
      Q23 = __ffma2_rn(b2, w23, Q23);
      if (AR && lite_ar_col<R>(c)) {
        const float g[4] = {fmaxf(w.x, 0.f), fmaxf(w.y, 0.f), fmaxf(w.z, 0.f), fmaxf(w.w, 0.f)};
        float2 ha, ha3, hb, hb3;
        ar_pow2(va, ha, ha3);
        ar_pow2(vb, hb, hb3);
#pragma unroll
        for (int k = 0; k < 4; k++) {
          const float2 gk = make_float2(g[k], g[k]), gr = make_float2(g[3 - k], g[3 - k]);
          HL[k] = __ffma2_rn(ha, gk, HL[k]);
          HL[k] = __ffma2_rn(hb, gr, HL[k]);
          HL3[k] = __ffma2_rn(ha3, gk, HL3[k]);
          HL3[k] = __ffma2_rn(hb3, gr, HL3[k]);
        }
      }
    }
    {
      constexpr int c = S / 2;  // even: the centre texel and the row's padding
      float4 w;
      if constexpr (H16) lut_pair_h16(p.lut_h, row + c, w, w_next);
      else w = __ldg(p.lut + row + c);
      const float v = get(c / N, c % N);
      const float2 v2 = make_float2(v, v);
      P01 = __ffma2_rn(v2, make_float2(w.x, w.y), P01);
      P23 = __ffma2_rn(v2, make_float2(w.z, w.w), P23);
      if (AR) {
        const float g[4] = {fmaxf(w.x, 0.f), fmaxf(w.y, 0.f), fmaxf(w.z, 0.f), fmaxf(w.w, 0.f)};
        float2 hc, hc3;
        ar_pow2(v, hc, hc3);
#pragma unroll
        for (int k = 0; k < 4; k++) {
          const float2 gk = make_float2(g[k], g[k]);
          HL[k] = __ffma2_rn(hc, gk, HL[k]);
          HL3[k] = __ffma2_rn(hc3, gk, HL3[k]);
        }
      }
    }
    float4 res = make_float4(P01.x + Q23.y, P01.y + Q23.x, P23.x + Q01.y, P23.y + Q01.x);
    const float4 hi = make_float4(HL[0].x, HL[1].x, HL[2].x, HL[3].x);
    const float4 lo = make_float4(HL[0].y, HL[1].y, HL[2].y, HL[3].y);
    const float4 hi2 = make_float4(HL3[0].x, HL3[1].x, HL3[2].x, HL3[3].x);
    const float4 lo2 = make_float4(HL3[0].y, HL3[1].y, HL3[2].y, HL3[3].y);
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
};

// --------------------------------------------------------------- ravu-3x --
template <int R, int CM, typename T, bool H16 = false, int TR = 8>
struct ThreeXTile {
  static constexpr int N = 2 * R - 1, S = N * N, HALO = R - 1;
  static constexpr int kRows = TR, kThreads = kTileW * TR;
  static constexpr bool kOutputTiles = false;
  static constexpr int TW = kTileW + N - 1, TH = TR + N - 1;
  static constexpr int C = CM == kLuma ? 1 : 3;
  static constexpr size_t smem_bytes = (size_t)(C + (CM == kRgb ? 1 : 0)) * TW * TH * 4;
  static constexpr int kPlanes = C;
  static constexpr int kMaxRegs = 0;  // the compiler's own allocation
  using Elem = T;

  __device__ static void run(const RavuArgs& p, int x0, int y0, float* smem, TmaCtx* tma = nullptr) {
    float* tile = smem;
    float* ltile = smem + C * TW * TH;
    if (!stage_frame<CM, TW, TH, kThreads, T>(p, tma, x0 - HALO, y0 - HALO, tile, ltile)) return;
    __syncthreads();
    const int tx = threadIdx.x % kTileW, ty = threadIdx.x / kTileW;
    const int gx = x0 + tx, gy = y0 + ty;
    if (gx >= p.W || gy >= p.H) return;
    auto val = [&](int c, int t) { return tile[c * TW * TH + (ty + t % N) * TW + tx + t / N]; };
    auto lum = [&](int kx, int ky) {
      return CM == kRgb ? ltile[(ty + ky) * TW + tx + kx] : tile[(ty + ky) * TW + tx + kx];
    };
    float a, b, d;
    structure_tensor<N, false>(lum, p.kp, a, b, d);
    const int key = ravu_key(a, b, d, p.kp);
    if (p.keys) p.keys[(size_t)gy * p.W + gx] = key;
    // 3x rows hold 2 * ceil(S / 2) texels: even, so the FP32 texel pairs are
    // 32-byte aligned without padding (1.2x over two 16-byte loads)
    const size_t row = (size_t)min(max(key, 0), p.lut_rows - 1) * (H16 ? p.lut_h_pitch : p.lut_cols);
    // res0 += a*w0 + b*w1.wzyx; res1 += a*w1 + b*w0.wzyx, as FP32x2 sums
    // P0 = sum a*w0, P1 = sum a*w1, Q0 = sum b*w0, Q1 = sum b*w1 (pairs .xy, .zw)
    float2 P0[C][2], P1[C][2], Q0[C][2], Q1[C][2];
#pragma unroll
    for (int c = 0; c < C; c++)
#pragma unroll
      for (int h = 0; h < 2; h++) P0[c][h] = P1[c][h] = Q0[c][h] = Q1[c][h] = make_float2(0.f, 0.f);
#pragma unroll
    for (int t = 0; t < S / 2; t++) {
      float4 w0, w1;
      if constexpr (H16) lut_pair_h16(p.lut_h, row + 2 * t, w0, w1);
      else lut_pair_f32(p.lut, row + 2 * t, w0, w1);
      const float2 w0a = make_float2(w0.x, w0.y), w0b = make_float2(w0.z, w0.w);
      const float2 w1a = make_float2(w1.x, w1.y), w1b = make_float2(w1.z, w1.w);
#pragma unroll
      for (int c = 0; c < C; c++) {
        const float va = val(c, t), vb = val(c, S - 1 - t);
        const float2 a2 = make_float2(va, va), b2 = make_float2(vb, vb);
        P0[c][0] = __ffma2_rn(a2, w0a, P0[c][0]);
        P0[c][1] = __ffma2_rn(a2, w0b, P0[c][1]);
        P1[c][0] = __ffma2_rn(a2, w1a, P1[c][0]);
        P1[c][1] = __ffma2_rn(a2, w1b, P1[c][1]);
        Q0[c][0] = __ffma2_rn(b2, w0a, Q0[c][0]);
        Q0[c][1] = __ffma2_rn(b2, w0b, Q0[c][1]);
        Q1[c][0] = __ffma2_rn(b2, w1a, Q1[c][0]);
        Q1[c][1] = __ffma2_rn(b2, w1b, Q1[c][1]);
      }
    }
    constexpr int tc = S / 2;
    float4 w0, w1;
    if constexpr (H16) lut_pair_h16(p.lut_h, row + 2 * tc, w0, w1);
    else lut_pair_f32(p.lut, row + 2 * tc, w0, w1);
    float4 r0[C], r1[C];
#pragma unroll
    for (int c = 0; c < C; c++) {
      const float v = val(c, tc);
      const float2 v2 = make_float2(v, v);
      P0[c][0] = __ffma2_rn(v2, make_float2(w0.x, w0.y), P0[c][0]);
      P0[c][1] = __ffma2_rn(v2, make_float2(w0.z, w0.w), P0[c][1]);
      P1[c][0] = __ffma2_rn(v2, make_float2(w1.x, w1.y), P1[c][0]);
      P1[c][1] = __ffma2_rn(v2, make_float2(w1.z, w1.w), P1[c][1]);
      // r0 = P0 + Q1.wzyx, r1 = P1 + Q0.wzyx
      r0[c] = make_float4(P0[c][0].x + Q1[c][1].y, P0[c][0].y + Q1[c][1].x, P0[c][1].x + Q1[c][0].y,
                          P0[c][1].y + Q1[c][0].x);
      r1[c] = make_float4(P1[c][0].x + Q0[c][1].y, P1[c][0].y + Q0[c][1].x, P1[c][1].x + Q0[c][0].y,
                          P1[c][1].y + Q0[c][0].x);
      const float4 a0 = make_float4(clampf(r0[c].x, 0.f, 1.f), clampf(r0[c].y, 0.f, 1.f),
                                    clampf(r0[c].z, 0.f, 1.f), clampf(r0[c].w, 0.f, 1.f));
      const float4 a1 = make_float4(clampf(r1[c].x, 0.f, 1.f), clampf(r1[c].y, 0.f, 1.f),
                                    clampf(r1[c].z, 0.f, 1.f), clampf(r1[c].w, 0.f, 1.f));
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
};

// The ravu keyed filter of one key evaluation: res[c] = sum over the S/2
// mirrored tap pairs of (x_i + x_{S-1-i}) * w_i (ravu-r3.hook:126-146), the
// weights w_i packed 4 to a texel.  Two tap pairs per FP32x2 FADD/FFMA.
template <int S, int C, class Val>
__device__ __forceinline__ void ravu_filter(const float4* L, const Val& val, float (&res)[C]) {
  float2 acc[C];
#pragma unroll
  for (int c = 0; c < C; c++) acc[c] = make_float2(0.0f, 0.0f);
#pragma unroll
  for (int q = 0; q < (S / 2 + 3) / 4; q++) {
    const float4 w4 = __ldg(L + q);
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int i0 = 4 * q + 2 * h, i1 = i0 + 1;
      const float2 w2 = h == 0 ? make_float2(w4.x, w4.y) : make_float2(w4.z, w4.w);
      if (i1 < S / 2) {
#pragma unroll
        for (int c = 0; c < C; c++) {
          const float2 s2 = __fadd2_rn(make_float2(val(c, i0), val(c, i1)),
                                       make_float2(val(c, S - 1 - i0), val(c, S - 1 - i1)));
          acc[c] = __ffma2_rn(s2, w2, acc[c]);
        }
      } else if (i0 < S / 2) {
#pragma unroll
        for (int c = 0; c < C; c++) acc[c].x = fmaf(val(c, i0) + val(c, S - 1 - i0), w2.x, acc[c].x);
      }
    }
  }
#pragma unroll
  for (int c = 0; c < C; c++) res[c] = acc[c].x + acc[c].y;
}

// ------------------------------------------------------ ravu lattice -----
// int11: the keyed filter over the input window (ravu-r3.hook:15-146).  Each
// thread stores its pixel's int11 value into the compact FP32 int11 plane
// (p.i11, [C][H][W]): one coalesced 4-byte store per channel.  The lattice
// program below writes every output pixel.
template <int R, int CM, typename T, int TR = 8>
struct Int11Tile {
  static constexpr int N = 2 * R, S = N * N, HALO = R - 1;
  static constexpr int kRows = TR, kThreads = kTileW * TR;
  static constexpr bool kOutputTiles = false;
  static constexpr int TW = kTileW + N - 1, TH = TR + N - 1;
  static constexpr int C = CM == kLuma ? 1 : 3;
  static constexpr size_t smem_bytes = (size_t)(C + (CM == kRgb ? 1 : 0)) * TW * TH * 4;
  static constexpr int kPlanes = C;
  // register caps measured best on GB300: r3 40 registers (6 CTAs of 8 rows
  // per SM; 32 registers spill the packed structure tensor), r4 48, r2 the
  // compiler's own allocation
  static constexpr int kMaxRegs = R == 3 ? 40 : (R == 4 ? 48 : 0);
  using Elem = T;

  __device__ static void run(const RavuArgs& p, int x0, int y0, float* smem, TmaCtx* tma = nullptr) {
    float* tile = smem;
    float* ltile = smem + C * TW * TH;
    if (!stage_frame<CM, TW, TH, kThreads, T>(p, tma, x0 - HALO, y0 - HALO, tile, ltile)) return;
    __syncthreads();
    const int tx = threadIdx.x % kTileW, ty = threadIdx.x / kTileW;
    const int gx = x0 + tx, gy = y0 + ty;
    if (gx >= p.W || gy >= p.H) return;
    auto val = [&](int c, int i) { return tile[c * TW * TH + (ty + i % N) * TW + tx + i / N]; };
    auto lum = [&](int kx, int ky) {
      return CM == kRgb ? ltile[(ty + ky) * TW + tx + kx] : tile[(ty + ky) * TW + tx + kx];
    };
    float a, b, d;
    structure_tensor<N, true>(lum, p.kp, a, b, d);
    const int key = ravu_key(a, b, d, p.kp);
    if (p.keys) p.keys[(size_t)gy * p.W + gx] = key;
    const float4* L = p.lut + (size_t)min(max(key, 0), p.lut_rows - 1) * p.lut_cols;
    float res[C];
    ravu_filter<S, C>(L, val, res);
    const size_t plane = (size_t)p.W * p.H;
#pragma unroll
    for (int c = 0; c < C; c++) {
      float v = clampf(res[c], 0.f, 1.f);
      if (p.i11_half) v = __half2float(__float2half_rn(v));
      p.i11[c * plane + (size_t)gy * p.W + gx] = v;
    }
  }
};

// Where lattice sample k (grid (k/N, k%N)) of an int10 (L=0) or int01 (L=1)
// pass reads: 0 = input, 1 = int11, at offsets (dx, dy).  The window is the
// 45-degree lattice: s = kx+ky-(N-1), d = ky-kx (ravu-r3.hook:155-189 int10,
// :289-323 int01).
template <int N>
__host__ __device__ constexpr int lat_src(int k, int L) {
  return (((k / N + k % N - (N - 1)) % 2 != 0) == (L == 0)) ? 0 : 1;
}
template <int N>
__host__ __device__ constexpr int lat_dx(int k, int L) {
  // int10: input (s+1)/2, int11 s/2; int01: input s/2, int11 (s-1)/2
  return L == 0 ? (lat_src<N>(k, L) == 0 ? (k / N + k % N - (N - 1) + 1) / 2 : (k / N + k % N - (N - 1)) / 2)
                : (lat_src<N>(k, L) == 0 ? (k / N + k % N - (N - 1)) / 2 : (k / N + k % N - (N - 1) - 1) / 2);
}
template <int N>
__host__ __device__ constexpr int lat_dy(int k, int L) {
  // int10: input d/2, int11 (d-1)/2; int01: input (d+1)/2, int11 d/2
  return L == 0 ? (lat_src<N>(k, L) == 0 ? (k % N - k / N) / 2 : (k % N - k / N - 1) / 2)
                : (lat_src<N>(k, L) == 0 ? (k % N - k / N + 1) / 2 : (k % N - k / N) / 2);
}

// int10 + int01: both lattice filters per input pixel (ravu-r3.hook:148-437).
// The input tile and the int11 tile (from the FP32 int11 plane, clamped to
// its edge: the clamp-to-edge of the int11 texture) are staged; each thread
// then holds all four samples of its output 2x2 block -- input (0,0), int10
// (1,0), int01 (0,1), int11 (1,1) -- and writes them as two pixel-pair rows.
template <int R, int CM, typename T, int TR = 8>
struct LatticeTile {
  static constexpr int N = 2 * R, S = N * N;
  static constexpr int kRows = TR, kThreads = kTileW * TR;
  static constexpr bool kOutputTiles = false;
  static constexpr int TW = kTileW + N - 1, TH = TR + N - 1;
  static constexpr int C = CM == kLuma ? 1 : 3;
  static constexpr int PL = C + (CM == kRgb ? 1 : 0);  // planes per tile set
  static constexpr size_t smem_bytes = (size_t)2 * PL * TW * TH * 4;
  static constexpr int kPlanes = C;
  // register caps measured best on GB300: r3 48 registers (5 CTAs of 8 rows
  // per SM), r4 80 (3), r2 the compiler's own allocation
  static constexpr int kMaxRegs = R == 3 ? 48 : (R == 4 ? 80 : 0);
  using Elem = T;

  __device__ static void run(const RavuArgs& p, int x0, int y0, float* smem, TmaCtx* tma = nullptr) {
    float* tin = smem;                      // input, offsets -(R-1) .. R
    float* lin = tin + C * TW * TH;
    float* t11 = smem + PL * TW * TH;       // int11, offsets -R .. R-1
    float* l11 = t11 + C * TW * TH;
    if (!stage_frame<CM, TW, TH, kThreads, T>(p, tma, x0 - (R - 1), y0 - (R - 1), tin, lin)) return;
    const size_t plane = (size_t)p.W * p.H;
    for (int i = threadIdx.x; i < TW * TH; i += kThreads) {
      const int ty = i / TW, tx = i % TW;
      const int cx = clampi(x0 - R + tx, 0, p.W - 1), cy = clampi(y0 - R + ty, 0, p.H - 1);
      float v[3] = {0.f, 0.f, 0.f};
#pragma unroll
      for (int c = 0; c < C; c++) {
        v[c] = __ldg(p.i11 + c * plane + (size_t)cy * p.W + cx);
        t11[c * TW * TH + i] = v[c];
      }
      if (CM == kRgb) l11[i] = rgb_luma(v[0], v[1], v[2]);
    }
    __syncthreads();
    const int tx = threadIdx.x % kTileW, ty = threadIdx.x / kTileW;
    const int gx = x0 + tx, gy = y0 + ty;
    if (gx >= p.W || gy >= p.H) return;
    float res[2][C];
#pragma unroll
    for (int L = 0; L < 2; L++) {
      auto idx = [&](int k) {
        return lat_src<N>(k, L) == 0 ? (ty + lat_dy<N>(k, L) + R - 1) * TW + tx + lat_dx<N>(k, L) + R - 1
                                     : (ty + lat_dy<N>(k, L) + R) * TW + tx + lat_dx<N>(k, L) + R;
      };
      auto val = [&](int c, int k) { return (lat_src<N>(k, L) == 0 ? tin : t11)[c * TW * TH + idx(k)]; };
      auto lum = [&](int kx, int ky) {
        const int k = kx * N + ky;
        if (CM != kRgb) return val(0, k);
        return (lat_src<N>(k, L) == 0 ? lin : l11)[idx(k)];
      };
      float a, b, d;
      structure_tensor<N, true>(lum, p.kp, a, b, d);
      const int key = ravu_key(a, b, d, p.kp);
      if (p.keys) p.keys[(size_t)(1 + L) * p.W * p.H + (size_t)gy * p.W + gx] = key;
      const float4* Lr = p.lut + (size_t)min(max(key, 0), p.lut_rows - 1) * p.lut_cols;
      ravu_filter<S, C>(Lr, val, res[L]);
    }
#pragma unroll
    for (int c = 0; c < C; c++) {
      T* o = static_cast<T*>(p.out[c]) + (size_t)(2 * gy) * p.out_pitch[c] + 2 * gx;
      // row 2i: input, int10; row 2i+1: int01, int11 (ravu-r3.hook:424-437)
      stp2(o, tin[c * TW * TH + (ty + R - 1) * TW + tx + R - 1], clampf(res[0][c], 0.f, 1.f));
      stp2(o + p.out_pitch[c], clampf(res[1][c], 0.f, 1.f), t11[c * TW * TH + (ty + R) * TW + tx + R]);
    }
  }
};

// ------------------------------------------------------------ ravu-zoom ---
struct ZoomPos {
  int i;    // floor(pos - 0.5)
  float s;  // fract(pos - 0.5)
};

// pos - 0.5 = ((2X+1) W - OW) / (2 OW), taken exactly (centre-aligned map).
__device__ __forceinline__ ZoomPos zoom_pos(int X, int W, int OW) {
  const long long num = (2LL * X + 1) * W - OW;
  const long long den = 2LL * OW;
  const long long q = num >= 0 ? num / den : -((-num + den - 1) / den);
  return {(int)q, (float)(num - q * den) / (float)den};
}

// Bilinear (FILTER LINEAR) fetch of one LUT texel at block column `blk` and
// sub-position (sx, sy) of key block `key`: x = blk*9 + 8 sx, y = key*9 + 8 sy
// (LUTPOS(x, 9) / (blocks, 288), ravu-zoom-r2.hook:23-31); clamp-to-edge.
// With q > 0 the fractions are rounded to multiples of 1/q, as a texture
// unit's fixed-point filter weights are (q = 256: 8 fractional bits).
template <bool H16>
__device__ __forceinline__ float4 lut_bilinear(const float4* lut, const uint2* luth, int hpitch, int rows, int cols,
                                               int key, int blk, float sx, float sy, float q) {
  const int pitch = H16 ? hpitch : cols;  // texels per stored row
  const float fx8 = 8.0f * sx, fy8 = 8.0f * sy;
  const float x0f = floorf(fx8), y0f = floorf(fy8);
  float fx = fx8 - x0f, fy = fy8 - y0f;
  if (q > 0.0f) {
    fx = rintf(fx * q) / q;
    fy = rintf(fy * q) / q;
  }
  const int xa = min(blk * 9 + (int)x0f, cols - 1), xb = min(xa + 1, cols - 1);
  const int ya = clampi(key * 9 + (int)y0f, 0, rows - 1), yb = min(ya + 1, rows - 1);
  const float4 v00 = lut_texel<H16>(lut, luth, (size_t)ya * pitch + xa);
  const float4 v01 = lut_texel<H16>(lut, luth, (size_t)ya * pitch + xb);
  const float4 v10 = lut_texel<H16>(lut, luth, (size_t)yb * pitch + xa);
  const float4 v11 = lut_texel<H16>(lut, luth, (size_t)yb * pitch + xb);
  const float gx = 1.0f - fx, gy = 1.0f - fy;
  float4 r;
  r.x = (v00.x * gx + v01.x * fx) * gy + (v10.x * gx + v11.x * fx) * fy;
  r.y = (v00.y * gx + v01.y * fx) * gy + (v10.y * gx + v11.y * fx) * fy;
  r.z = (v00.z * gx + v01.z * fx) * gy + (v10.z * gx + v11.z * fx) * fy;
  r.w = (v00.w * gx + v01.w * fx) * gy + (v10.w * gx + v11.w * fx) * fy;
  return r;
}

__device__ __forceinline__ float comp4(const float4& v, int i) {
  return i == 0 ? v.x : (i == 1 ? v.y : (i == 2 ? v.z : v.w));
}

// One thread per OUTPUT pixel; the tile is 32 x TR output pixels and stages the
// input rectangle they touch (at most (32+N+1) x (TR+N+1) when upscaling;
// its origin follows from the tile's source positions, as the compute
// shader's rect, compute/ravu-zoom-ar-r2.hook:28-37): by clamped loads, or
// (TMA staging, interior rectangles) from one TMA box per plane whose size
// the host fits to the launch's scale factor (tma_box_of), converting just
// the rectangle.
template <int R, int CM, bool AR, typename T, bool H16 = false, int TR = 8>
struct ZoomTile {
  static constexpr int N = 2 * R, S = N * N, LO = R - 1;
  static constexpr int kRows = TR, kThreads = kTileW * TR;
  static constexpr bool kOutputTiles = true;
  static constexpr int RW = kTileW + N + 1, RH = TR + N + 1;
  static constexpr int C = CM == kLuma ? 1 : 3;
  static constexpr int NB = (S / 2 + 3) / 4;  // LUT texels per half window
  // input rectangle planes, then the source positions of the tile's 32
  // columns and TR rows
  static constexpr size_t smem_bytes =
      (size_t)(C + (CM == kRgb ? 1 : 0)) * RW * RH * 4 + (kTileW + TR) * sizeof(ZoomPos);

  static constexpr int kPlanes = C;
  static constexpr int kMaxRegs = 0;  // the compiler's own allocation
  // the largest TMA box: the largest rectangle plus up to 7 lead columns
  static constexpr int kBoxMaxW = (RW + 7 + 7) & ~7, kBoxMaxH = RH;
  using Elem = T;

  __device__ static void run(const RavuArgs& p, int X0, int Y0, float* smem, TmaCtx* tma = nullptr) {
    float* tile = smem;
    float* ltile = smem + C * RW * RH;
    ZoomPos* pos = reinterpret_cast<ZoomPos*>(smem + (C + (CM == kRgb ? 1 : 0)) * RW * RH);
    const int X1 = min(X0 + kTileW - 1, p.OW - 1), Y1 = min(Y0 + TR - 1, p.OH - 1);
    static_assert(kThreads >= kTileW + TR, "one thread per tile column and row");
    if (threadIdx.x < kTileW + TR) {  // one exact position per tile column / row
      const int t = threadIdx.x;
      pos[t] = t < kTileW ? zoom_pos(min(X0 + t, X1), p.W, p.OW) : zoom_pos(min(Y0 + t - kTileW, Y1), p.H, p.OH);
    }
    __syncthreads();
    const int rx = pos[0].i - LO, ry = pos[kTileW].i - LO;
    const int rw = pos[X1 - X0].i + R - rx + 1, rh = pos[kTileW + Y1 - Y0].i + R - ry + 1;
    if (rw > RW || rh > RH) {  // only reachable when downscaling, which the host rejects
      if (threadIdx.x == 0 && p.err) atomicCAS(p.err, 0, kErrTileOverflow);
      return;
    }
    // every operand of these tests is uniform across the CTA
    int staged = 0;
    if (tma && tma->map && !tma->dead && rx >= 0 && ry >= 0 && rx + rw <= p.W && ry + rh <= p.H &&
        (rx & 7) + rw <= p.box_w && rh <= p.box_h) {
      const uint32_t pb = ((uint32_t)p.box_w * p.box_h * sizeof(T) + 127u) & ~127u;
      staged = tma_stage_box<CM, kThreads, T>(p, tma, rx & ~7, ry, p.box_w, p.box_h, pb, rx & 7, rw, rh, RW,
                                              RW * RH, tile, ltile);
      if (staged < 0) return;
    }
    for (int i = threadIdx.x; !staged && i < rw * rh; i += kThreads) {
      const int ty = i / rw, tx = i % rw;
      const int gx = clampi(rx + tx, 0, p.W - 1), gy = clampi(ry + ty, 0, p.H - 1);
      float v[3] = {0.f, 0.f, 0.f};
#pragma unroll
      for (int c = 0; c < C; c++) {
        v[c] = ldp(static_cast<const T*>(p.in[c]) + (size_t)gy * p.in_pitch[c] + gx);
        tile[c * RW * RH + ty * RW + tx] = v[c];
      }
      if (CM == kRgb) ltile[ty * RW + tx] = rgb_luma(v[0], v[1], v[2]);
    }
    __syncthreads();
    const int X = X0 + threadIdx.x % kTileW, Y = Y0 + threadIdx.x / kTileW;
    if (X >= p.OW || Y >= p.OH) return;
    const ZoomPos px = pos[threadIdx.x % kTileW], py = pos[kTileW + threadIdx.x / kTileW];
    const int bx = px.i - LO - rx, by = py.i - LO - ry;  // window origin in the tile
    auto val = [&](int c, int k) { return tile[c * RW * RH + (by + k % N) * RW + bx + k / N]; };
    auto lum = [&](int kx, int ky) {
      return CM == kRgb ? ltile[(by + ky) * RW + bx + kx] : tile[(by + ky) * RW + bx + kx];
    };
    float a, b, d;
    structure_tensor<N, true>(lum, p.kp, a, b, d);
    const int key = ravu_key(a, b, d, p.kp);  // no +0.5 row centring (ravu-zoom-r2.hook:124)
    if (p.keys) p.keys[(size_t)Y * p.OW + X] = key;
    const float sx = px.s, sy = py.s, ix = 1.0f - sx, iy = 1.0f - sy;
    // anti-ringing sums per channel as FP32x2 pairs (hi, lo) and (hi2, lo2)
    float res[C];
    float2 HL[C], HL3[C];
#pragma unroll
    for (int c = 0; c < C; c++) {
      res[c] = 0.0f;
      HL[c] = HL3[c] = make_float2(0.0f, 0.0f);
    }
#pragma unroll
    for (int blk = 0; blk < NB; blk++) {
      const float4 ws = lut_bilinear<H16>(p.lut, p.lut_h, p.lut_h_pitch, p.lut_rows, p.lut_cols, key, blk, sx, sy, p.lut_frac);
      const float4 wi = lut_bilinear<H16>(p.lut, p.lut_h, p.lut_h_pitch, p.lut_rows, p.lut_cols, key, blk, ix, iy, p.lut_frac);
      float4 as = make_float4(0.f, 0.f, 0.f, 0.f), ai = as;
      if (AR) {  // the anti-ringing LUT stays FP32 in every form but mpv's (most of
                 // its values lie below FP16's normal range)
        as = lut_bilinear<false>(p.lut_ar, nullptr, 0, p.lut_rows, p.lut_cols, key, blk, sx, sy, p.lut_frac);
        ai = lut_bilinear<false>(p.lut_ar, nullptr, 0, p.lut_rows, p.lut_cols, key, blk, ix, iy, p.lut_frac);
      }
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const int i = blk * 4 + j;
        if (i < S / 2) {
          const int k2 = S - 1 - i;
#pragma unroll
          for (int c = 0; c < C; c++) {
            const float va = val(c, i), vb = val(c, k2);
            res[c] += va * comp4(ws, j);
            res[c] += vb * comp4(wi, j);
            if (AR) {
              float2 pa, pa3, pb, pb3;
              ar_pow2(va, pa, pa3);
              ar_pow2(vb, pb, pb3);
              const float2 wa = make_float2(comp4(as, j), comp4(as, j));
              const float2 wb = make_float2(comp4(ai, j), comp4(ai, j));
              HL[c] = __ffma2_rn(pa, wa, HL[c]);
              HL[c] = __ffma2_rn(pb, wb, HL[c]);
              HL3[c] = __ffma2_rn(pa3, wa, HL3[c]);
              HL3[c] = __ffma2_rn(pb3, wb, HL3[c]);
            }
          }
        }
      }
    }
#pragma unroll
    for (int c = 0; c < C; c++) {
      const float v = AR ? ar_finish(res[c], HL[c].y, HL[c].x, HL3[c].y, HL3[c].x, p.ar) : clampf(res[c], 0.f, 1.f);
      stp(static_cast<T*>(p.out[c]) + (size_t)Y * p.out_pitch[c] + X, v);
    }
  }
};

// One CTA per tile of a single frame; with TMA the frame tile of interior
// tiles comes in by cp.async.bulk.tensor.
template <class Prog, bool TMA>
__device__ __forceinline__ void tile_body(const RavuArgs& p, const TmaMaps& maps) {
  extern __shared__ __align__(128) float4 tile_smem[];
  float* smem = reinterpret_cast<float*>(tile_smem);
  if (TMA) {
    __shared__ __align__(8) unsigned long long mbar;
    if (threadIdx.x == 0) mbar_init(smem_u32(&mbar), 1);
    __syncthreads();
    TmaCtx ctx{maps.map, smem_u32(&mbar),
               reinterpret_cast<unsigned char*>(tile_smem) + ((Prog::smem_bytes + 127) & ~(size_t)127), 0u, 0};
    Prog::run(p, blockIdx.x * kTileW, blockIdx.y * Prog::kRows, smem, &ctx);
    tma_drain(&ctx);
  } else {
    Prog::run(p, blockIdx.x * kTileW, blockIdx.y * Prog::kRows, smem, nullptr);
  }
}

// Programs with kMaxRegs > 0 run under that register cap (the same cap at
// every tile height); the others keep the compiler's own allocation.
template <class Prog, bool TMA>
__global__ void __launch_bounds__(Prog::kThreads) tile_kernel(const __grid_constant__ RavuArgs p,
                                                              const __grid_constant__ TmaMaps maps) {
  tile_body<Prog, TMA>(p, maps);
}
template <class Prog, bool TMA>
__global__ void __maxnreg__(Prog::kMaxRegs) tile_kernel_mr(const __grid_constant__ RavuArgs p,
                                                           const __grid_constant__ TmaMaps maps) {
  tile_body<Prog, TMA>(p, maps);
}

template <class Prog, bool TMA>
void launch_tile_kernel(dim3 grid, size_t smem, cudaStream_t s, const RavuArgs& a, const TmaMaps& maps) {
  if constexpr (Prog::kMaxRegs > 0)
    tile_kernel_mr<Prog, TMA><<<grid, Prog::kThreads, smem, s>>>(a, maps);
  else
    tile_kernel<Prog, TMA><<<grid, Prog::kThreads, smem, s>>>(a, maps);
}

bool encode_plane_map(CUtensorMap* map, const void* base, int W, int H, int pitch, int dtype, int box_w,
                      int box_h);

// TMA boxes of a program.  The frame-tile programs have one fixed box (the
// tile and its halo plus up to 7 lead columns).  ravu-zoom's box holds the
// largest input rectangle of the launch's scale factor: n consecutive output
// columns span at most floor((n-1) W / OW) + 1 source steps, plus the 2R
// window (rows likewise), capped at the program's largest box; a tile whose
// rectangle does not fit stages by clamped loads.
template <class Prog>
constexpr int tma_box_max_w() {
  if constexpr (Prog::kOutputTiles) return Prog::kBoxMaxW;
  else return tma_box_w<Prog::TW>();
}
template <class Prog>
constexpr int tma_box_max_h() {
  if constexpr (Prog::kOutputTiles) return Prog::kBoxMaxH;
  else return Prog::TH;
}
template <class Prog>
void tma_box_of(const RavuArgs& a, int* bw, int* bh) {
  if constexpr (Prog::kOutputTiles) {
    const int w = (int)((long long)(kTileW - 1) * a.W / a.OW) + 1 + Prog::N;
    const int h = (int)((long long)(Prog::kRows - 1) * a.H / a.OH) + 1 + Prog::N;
    *bw = ((w + 7 + 7) & ~7) < Prog::kBoxMaxW ? ((w + 7 + 7) & ~7) : Prog::kBoxMaxW;
    *bh = h < Prog::kBoxMaxH ? h : Prog::kBoxMaxH;
  } else {
    *bw = tma_box_max_w<Prog>();
    *bh = tma_box_max_h<Prog>();
  }
}
// Shared memory of the landing area: one largest box per plane.
template <class Prog>
constexpr size_t tma_landing_bytes() {
  return (size_t)Prog::kPlanes *
         (((size_t)tma_box_max_w<Prog>() * tma_box_max_h<Prog>() * sizeof(typename Prog::Elem) + 127) & ~(size_t)127);
}
// The maps of a's input planes for Prog's box (recorded in a->box_w / box_h);
// false when a plane cannot be mapped (alignment, a box larger than the plane).
template <class Prog>
bool encode_tma(RavuArgs* a, TmaMaps* maps) {
  int bw, bh;
  tma_box_of<Prog>(*a, &bw, &bh);
  const int dt = sizeof(typename Prog::Elem) == 4 ? 0 : 1;
  for (int c = 0; c < Prog::kPlanes; c++)
    if (!encode_plane_map(&maps->map[c], a->in[c], a->W, a->H, a->in_pitch[c], dt, bw, bh)) return false;
  a->box_w = bw;
  a->box_h = bh;
  return true;
}

// One CTA per tile of the frame (of the output frame for output-tiled
// programs), staged by TMA when the frame asks for it and its planes map.
template <class Prog>
int launch_tiles(const RavuArgs& a, cudaStream_t s) {
  static_assert(Prog::smem_bytes <= 48 * 1024, "tile program needs more than the default shared memory");
  const int fw = Prog::kOutputTiles ? a.OW : a.W, fh = Prog::kOutputTiles ? a.OH : a.H;
  const int tiles_w = (fw + kTileW - 1) / kTileW, tiles_h = (fh + Prog::kRows - 1) / Prog::kRows;
  TmaMaps maps;
  std::memset(&maps, 0, sizeof maps);
  if constexpr (Prog::kPlanes > 0) {
    RavuArgs b = a;
    if (a.staging == 1 && encode_tma<Prog>(&b, &maps)) {
      constexpr size_t smem = ((Prog::smem_bytes + 127) & ~(size_t)127) + tma_landing_bytes<Prog>();
      static_assert(smem <= 48 * 1024, "TMA staging needs more than the default shared memory");
      launch_tile_kernel<Prog, true>(dim3(tiles_w, tiles_h), smem, s, b, maps);
      return 0;
    }
  }
  launch_tile_kernel<Prog, false>(dim3(tiles_w, tiles_h), Prog::smem_bytes, s, a, maps);
  return 0;
}

// ------------------------------------------------------ persistent batches ---
// Program ids of a batch job (tile program and form; see batch.cu).
enum ProgId : int {
  kLite0 = 0,      // + (R-2)*2 + AR
  kThreeX0 = 6,    // + (R-2)*3 + CM
  kInt110 = 15,    // + (R-2)*3 + CM
  kLattice0 = 24,  // + (R-2)*3 + CM
  kZoom0 = 33,     // + (R-2)*6 + CM*2 + AR
  kLiteH0 = 45,    // fast form (FP16 LUT texels): as kLite0
  kThreeXH0 = 51,  //   as kThreeX0
  kZoomH0 = 60,    //   as kZoom0
  kNumProgs = 72
};

// One batch job: a frame's arguments, its place in its launch's tile range
// and (has_maps) the TMA maps of its input planes, read by the TMA unit
// from global memory.
struct DevJob {
  RavuArgs a;
  int prog;
  int tiles_w;
  int first_tile;  // prefix sum within its launch group
  int has_maps;
  TmaMaps maps;    // 64-byte aligned (CUtensorMap)
};
// every job's maps start on a 64-byte boundary of the (256-byte aligned) table
static_assert(sizeof(DevJob) % 64 == 0 && offsetof(DevJob, maps) % 64 == 0, "tensor maps must be 64-byte aligned");

// Persistent CTAs of one tile program: claim tile numbers from `counter`
// until `total`; a tile's job is the last whose first tile <= the number
// (binary search over the group's prefix sums); the job's arguments are
// copied to shared memory when the job changes.  Every job of a launch runs
// the same program, so register use and shared memory are the program's own.
template <class Prog>
__device__ __forceinline__ void persistent_body(const DevJob* __restrict__ jobs, int n_jobs, int total,
                                                int* counter) {
  extern __shared__ __align__(128) float4 psmem[];
  float* smem = reinterpret_cast<float*>(psmem);
  __shared__ RavuArgs s_args;
  // TMA staging of interior tiles (jobs with maps; programs with planes):
  // the landing area follows the program's shared memory; the mbarrier is
  // initialised before the first claim barrier, which orders it before use
  __shared__ __align__(8) unsigned long long mbar;
  if (Prog::kPlanes > 0 && threadIdx.x == 0) mbar_init(smem_u32(&mbar), 1);
  TmaCtx ctx{nullptr, smem_u32(&mbar),
             reinterpret_cast<unsigned char*>(psmem) + ((Prog::smem_bytes + 127) & ~(size_t)127), 0u, 0};
  // claim slots alternate between iterations: thread 0 fills slot (i+1)&1
  // while the other threads may still read slot i&1, and cannot get two
  // iterations ahead (the claim barrier of iteration i+1 holds it)
  __shared__ int s_item[2], s_job[2], s_tw[2], s_first[2];
  int loaded = -1;
  // thread 0 claims the next tile while the current one runs
  int next = threadIdx.x == 0 ? atomicAdd(counter, 1) : 0;
  for (int it = 0;; it ^= 1) {
    if (threadIdx.x == 0) {
      const int item = next;
      s_item[it] = item;
      if (item < total) {
        next = atomicAdd(counter, 1);
        int lo = 0, hi = n_jobs - 1;  // last job whose first tile <= item
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (jobs[mid].first_tile <= item) lo = mid; else hi = mid - 1;
        }
        s_job[it] = lo;
        s_tw[it] = jobs[lo].tiles_w;
        s_first[it] = jobs[lo].first_tile;
      }
    }
    __syncthreads();
    const int item = s_item[it];
    if (item >= total) break;
    const int job = s_job[it], tw = s_tw[it], first = s_first[it];
    if (job != loaded) {  // uniform: every thread reads the same slot
      // every thread is past the previous tile (the claim barrier above), so
      // s_args is free
      loaded = job;
      const int* src = reinterpret_cast<const int*>(&jobs[loaded].a);
      int* dst = reinterpret_cast<int*>(&s_args);
      for (int i = threadIdx.x; i < (int)(sizeof(RavuArgs) / 4); i += Prog::kThreads) dst[i] = src[i];
      ctx.map = jobs[loaded].has_maps ? jobs[loaded].maps.map : nullptr;
      __syncthreads();
    }
    const int t = item - first;
    // No barrier after the tile: the next tile's staging and argument copy
    // come after the next claim barrier, which every thread reaches only
    // when done with this tile.
    Prog::run(s_args, (t % tw) * kTileW, (t / tw) * Prog::kRows, smem, Prog::kPlanes > 0 ? &ctx : nullptr);
  }
  tma_drain(&ctx);
}

template <class Prog>
__global__ void __launch_bounds__(Prog::kThreads) persistent_kernel(const DevJob* __restrict__ jobs, int n_jobs,
                                                                    int total, int* counter) {
  persistent_body<Prog>(jobs, n_jobs, total, counter);
}
template <class Prog>
__global__ void __maxnreg__(Prog::kMaxRegs) persistent_kernel_mr(const DevJob* __restrict__ jobs, int n_jobs,
                                                                 int total, int* counter) {
  persistent_body<Prog>(jobs, n_jobs, total, counter);
}

// Launch, occupancy query and TMA map encoding of one program's persistent
// kernel.
struct PersistentOps {
  void (*launch)(const DevJob* jobs, int n_jobs, int total, int* counter, int grid, cudaStream_t s);
  int (*fit)();                                // resident CTAs per SM
  bool (*encode)(RavuArgs* a, TmaMaps* maps);  // false: the job stages by clamped loads
};

// Shared memory of a persistent CTA: the program's, then (programs with
// planes) the TMA landing area of every plane.
template <class Prog>
constexpr size_t persistent_smem() {
  if constexpr (Prog::kPlanes > 0)
    return ((Prog::smem_bytes + 127) & ~(size_t)127) + tma_landing_bytes<Prog>();
  else
    return Prog::smem_bytes;
}

template <class Prog>
bool persistent_encode(RavuArgs* a, TmaMaps* maps) {
  if constexpr (Prog::kPlanes > 0) return encode_tma<Prog>(a, maps);
  else return false;
}

template <class Prog>
PersistentOps persistent_ops() {
  constexpr size_t kSmem = persistent_smem<Prog>();
  static_assert(kSmem <= 48 * 1024, "persistent tile program needs more than the default shared memory");
  static_assert(Prog::kRows == kBatchTileRows, "persistent batches number tiles of kBatchTileRows rows");
  if constexpr (Prog::kMaxRegs > 0) {
    return {[](const DevJob* j, int n, int total, int* c, int grid, cudaStream_t s) {
              persistent_kernel_mr<Prog><<<grid, Prog::kThreads, kSmem, s>>>(j, n, total, c);
            },
            []() {
              int fit = 0;
              cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, persistent_kernel_mr<Prog>, Prog::kThreads, kSmem);
              return fit;
            },
            persistent_encode<Prog>};
  } else {
    return {[](const DevJob* j, int n, int total, int* c, int grid, cudaStream_t s) {
              persistent_kernel<Prog><<<grid, Prog::kThreads, kSmem, s>>>(j, n, total, c);
            },
            []() {
              int fit = 0;
              cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, persistent_kernel<Prog>, Prog::kThreads, kSmem);
              return fit;
            },
            persistent_encode<Prog>};
  }
}

// The ops of program `prog` for plane dtype `dtype` (0 FP32, 1 FP16), or
// null members when `prog` is not the family's; defined beside the family's
// per-frame launchers.
PersistentOps persistent_ops_lite(int prog, int dtype);     // lite, 3x (ravu_lite.cu)
PersistentOps persistent_ops_lattice(int prog, int dtype);  // int11, lattice (ravu_lattice.cu)
PersistentOps persistent_ops_zoom(int prog, int dtype);     // zoom (ravu_zoom.cu)

}  // namespace pz
