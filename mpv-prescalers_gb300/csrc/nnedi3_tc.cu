// NNEDI3 doubling pass on the 5th-generation tensor cores (tcgen05).
//
// Reference arithmetic: nnedi3-nns16-win8x4.hook:20-50 (normalise the 8xK
// window, nns neuron pairs, exp-weighted Elliott blend); pass geometry as in
// the CUDA-core kernel (nnedi3_simt.cu).
//
// Per CTA tile of 128 interpolated pixels (4 warps x 32 consecutive pixels):
//   1. the window tile is staged in shared memory; each thread normalises its
//      pixel's window, x_hat = (x - mean) * invstd, and writes it as one FP16
//      row of the A operand [128 x T] (K-major, no-swizzle core matrices:
//      8 rows x 16 bytes, LBO = 128 B between K-neighbours, SBO = T*16 B
//      between 8-row groups);
//   2. one thread issues T/16 tcgen05.mma.kind::f16 instructions (M = 128,
//      N = 2*nns, or two N = 256 halves for nns256) against the resident
//      weight operand B [2*nns x T] (rows 0..nns-1: softmax branch, nns..:
//      Elliott branch), accumulating FP32 in tensor memory, and commits to an
//      mbarrier;
//   3. after the (time-bounded) mbarrier wait, warp w reads TMEM lanes
//      32w..32w+31 -- one lane per pixel -- with tcgen05.ld.32x32b.x32 and
//      runs the epilogue in FP32: s1 = D + mean*invstd*sum(A_k) + a_k,
//      e = exp(s1), s2 likewise, wsum += e, vsum += e * s2 / (1 + |s2|).
// The mean term restores <x, A_k> * invstd exactly (x_hat is centred).
// The CTA is persistent: weights and TMEM are set up once per CTA.
//
// Every mbarrier wait is bounded (kWaitNs of %globaltimer).  A wait that runs
// out ends the CTA's loop; before the tensor memory is freed, the issuing
// thread commits once more and waits (bounded again) until every MMA it has
// issued has completed, so no MMA can still write the freed columns; the
// failure is reported as kErrWaitTimeout in the device error word.
#include "async.cuh"
#include "kernels.h"

namespace pz {
namespace {

constexpr int kThreads = 128;  // 4 warps, one TMEM lane quarter each

// tcgen05 shared-memory matrix descriptor, no swizzle, K-major.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version for tcgen05
  return d;                // base offset 0, relative LBO, layout 0 = no swizzle
}

// Instruction descriptor, kind::f16: D = F32, A = B = F16, both K-major.
__host__ __device__ constexpr uint32_t instr_desc(int M, int N) {
  return (1u << 4) | (0u << 7) | (0u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_f16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
               : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[32]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ float exp2f_approx(float x) {
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Neurons are processed in chunks of NC (32, or 16 for nns16): chunk k's
// accumulator holds NC softmax-branch and NC Elliott-branch columns, and two
// chunk buffers alternate in tensor memory (4*NC columns per CTA), so up to
// four CTAs share an SM's 512 columns.  The MMA of chunk k+2 is issued as
// soon as every warp has read chunk k, and runs under chunk k's epilogue.
// Operand B is stored chunk-major: rows [2*NC*k, 2*NC*k + NC) are the
// softmax weights of neurons k*NC.., the next NC rows their Elliott weights.
template <int WH, int NNS, bool XP, typename T>
__global__ void __launch_bounds__(kThreads) nn_tc_kernel(const __grid_constant__ NnArgs p) {
  constexpr int NT = 8 * WH;                 // window taps
  constexpr int KP = (NT + 3 + 15) / 16 * 16;  // K: taps, mean term, bias hi/lo, zero pad
  constexpr int NC = NNS < 32 ? NNS : 32;    // neurons per chunk
  constexpr int NCH = NNS / NC;              // chunks per tile
  constexpr int CCOL = 2 * NC;               // TMEM columns per chunk buffer
  constexpr int TCOLS = 2 * CCOL;            // two buffers
  constexpr int DY0 = -(WH / 2 - 1);
  constexpr int OX0 = XP ? DY0 : -3, OX1 = XP ? WH / 2 : 4;
  constexpr int OY0 = XP ? -3 : DY0, OY1 = XP ? 4 : WH / 2;
  constexpr int TW = 32 + OX1 - OX0, TH = 4 + OY1 - OY0;
  constexpr uint32_t SBO = KP * 16;          // bytes between 8-row groups (A and B)
  constexpr uint32_t LBO = 128;              // bytes between K-adjacent core matrices
  static_assert(NNS % NC == 0 && NC % 16 == 0, "neuron count must be a multiple of 16");

  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char* sB = smem;                                    // [2*NNS x KP] f16
  unsigned char* sA = sB + 2 * NNS * KP * 2;                   // [128 x KP] f16
  float* tile = reinterpret_cast<float*>(sA + 128 * KP * 2);   // [TH][TW]
  __shared__ __align__(8) unsigned long long mbar[3];  // two chunk buffers, drain
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  {  // one-time setup: the weight operand
    const uint4* src = reinterpret_cast<const uint4*>(p.wts_h);
    uint4* dst = reinterpret_cast<uint4*>(sB);
    for (int i = tid; i < 2 * NNS * KP * 2 / 16; i += kThreads) dst[i] = __ldg(src + i);
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(TCOLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    mbar_init(smem_u32(&mbar[0]), 1);
    mbar_init(smem_u32(&mbar[1]), 1);
    mbar_init(smem_u32(&mbar[2]), 1);
    abort_flag = 0;
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base;
  const uint32_t mb0 = smem_u32(&mbar[0]), mb1 = smem_u32(&mbar[1]);
  const uint32_t a_addr = smem_u32(sA), b_addr = smem_u32(sB);
  constexpr uint32_t IDESC = instr_desc(128, CCOL);
  // D[buf] (+)= A x B[chunk]^T over the whole K; completion on mbar[buf]
  auto issue_chunk = [&](int chunk, int buf) {
#pragma unroll
    for (int ks = 0; ks < KP / 16; ks++) {
      const uint64_t ad = smem_desc(a_addr + ks * 2 * LBO, LBO, SBO);
      const uint64_t bd = smem_desc(b_addr + (uint32_t)chunk * (CCOL / 8) * SBO + ks * 2 * LBO, LBO, SBO);
      mma_f16(tmem + buf * CCOL, ad, bd, IDESC, ks > 0 ? 1u : 0u);
    }
    mma_commit(buf ? mb1 : mb0);
  };

  const T* in = static_cast<const T*>(p.in);
  T* out = static_cast<T*>(p.out);
  const int tiles_x = (p.W + 31) / 32, tiles_y = (p.H + 3) / 4;
  const int ntiles = tiles_x * tiles_y;
  uint32_t phase = 0;  // bit b: parity of mbar[b]'s next phase

  // the window tile of the next tile is loaded into registers while the
  // current tile's neurons run (at most PF values per thread)
  constexpr int PF = (TW * TH + kThreads - 1) / kThreads;
  float pre[PF];
  auto prefetch = [&](int tid_) {
    if (tid_ >= ntiles) return;
    const int px0 = (tid_ % tiles_x) * 32, py0 = (tid_ / tiles_x) * 4;
#pragma unroll
    for (int r = 0; r < PF; r++) {
      const int i = tid + r * kThreads;
      if (i < TW * TH) {
        const int ty = i / TW, tx = i % TW;
        const int gx = clampi(px0 + OX0 + tx, 0, p.W - 1), gy = clampi(py0 + OY0 + ty, 0, p.H - 1);
        pre[r] = ldp(in + (size_t)gy * p.in_pitch + gx);
      }
    }
  };
  prefetch(blockIdx.x);
  for (int tile_id = blockIdx.x; tile_id < ntiles; tile_id += gridDim.x) {
    const int x0 = (tile_id % tiles_x) * 32, y0 = (tile_id / tiles_x) * 4;
#pragma unroll
    for (int r = 0; r < PF; r++) {
      const int i = tid + r * kThreads;
      if (i < TW * TH) tile[i] = pre[r];
    }
    __syncthreads();
    // ---- normalise this thread's window into its A row (pixel m = tid)
    // The sums run as 8 independent partial sums (one per window column):
    // the window's loads and adds form no serial chain of NT steps.
    const int m = tid, px = lane, py = warp;
    float xv[NT];
#pragma unroll
    for (int t = 0; t < NT; t++) {
      const int dx = t % 8 - 3, dy = t / 8 + DY0;
      const int ox = XP ? dy : dx, oy = XP ? dx : dy;
      xv[t] = tile[(py + oy - OY0) * TW + px + ox - OX0];
    }
    float ps[8];
#pragma unroll
    for (int c = 0; c < 8; c++) ps[c] = xv[c];
#pragma unroll
    for (int t = 8; t < NT; t++) ps[t % 8] += xv[t];
    const float mean = (((ps[0] + ps[1]) + (ps[2] + ps[3])) + ((ps[4] + ps[5]) + (ps[6] + ps[7]))) * (1.0f / NT);
#pragma unroll
    for (int c = 0; c < 8; c++) {
      const float d = xv[c] - mean;
      ps[c] = d * d;
    }
#pragma unroll
    for (int t = 8; t < NT; t++) {
      const float d = xv[t] - mean;
      ps[t % 8] = fmaf(d, d, ps[t % 8]);
    }
    const float var = (((ps[0] + ps[1]) + (ps[2] + ps[3])) + ((ps[4] + ps[5]) + (ps[6] + ps[7]))) * (1.0f / NT);
    const float invstd = var >= kFltEps ? rsqrtf(var) : 0.0f;
    const float stdv = var * invstd;
    const float orig = tile[(py - OY0) * TW + px - OX0];
    {  // A row: [x_hat (NT), mean * invstd, 1, 1, 0...], x_hat = x * invstd - mean * invstd
      unsigned char* row = sA + (m >> 3) * SBO + (m & 7) * 16;
      const float mterm = mean * invstd;
#pragma unroll
      for (int kc = 0; kc < KP / 8; kc++) {
        __half2 h[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
          const int t = 8 * kc + 2 * j;
          const float v0 = t < NT ? fmaf(xv[t], invstd, -mterm) : (t == NT ? mterm : (t <= NT + 2 ? 1.0f : 0.0f));
          const float v1 = t + 1 < NT ? fmaf(xv[t + 1], invstd, -mterm)
                                      : (t + 1 == NT ? mterm : (t + 1 <= NT + 2 ? 1.0f : 0.0f));
          h[j] = __floats2half2_rn(v0, v1);
        }
        *reinterpret_cast<uint4*>(row + kc * LBO) = *reinterpret_cast<uint4*>(h);
      }
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (tid == 0) {
      issue_chunk(0, 0);
      if (NCH > 1) issue_chunk(1, 1);
    }
    prefetch(tile_id + gridDim.x);  // in flight during the epilogue
    // ---- epilogue: lane m of TMEM holds pixel m's pre-activations
    // (softmax branch already in log2 units, Elliott branch as is)
    float wsum = 0.0f, vsum = 0.0f;
    const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
    for (int k = 0; k < NCH; k++) {
      const int b = k & 1;
      if (!mbar_wait_bounded(b ? mb1 : mb0, (phase >> b) & 1u)) atomicExch(&abort_flag, 1);
      phase ^= 1u << b;
      tc_fence_after();
      float s1[32], s2[32];
      if (NC == 32) {
        tmem_ld32(lane_addr + b * CCOL, s1);
        tmem_ld32(lane_addr + b * CCOL + NC, s2);
      } else {
        tmem_ld16(lane_addr + b * CCOL, s1);
        tmem_ld16(lane_addr + b * CCOL + NC, s2);
      }
      tmem_wait_ld();
      tc_fence_before();
      __syncthreads();  // every warp has read buffer b
      if (abort_flag) break;
      if (tid == 0 && k + 2 < NCH) {
        tc_fence_after();
        issue_chunk(k + 2, b);
      }
#pragma unroll
      for (int j = 0; j < NC; j += 2) {
        const float b0 = s2[j], b1 = s2[j + 1];
        const float e0 = exp2f_approx(s1[j]), e1 = exp2f_approx(s1[j + 1]);
        // b/(1+|b|) for two neurons from one reciprocal of the product
        const float d0 = 1.0f + fabsf(b0), d1 = 1.0f + fabsf(b1);
        const float r = __fdividef(1.0f, d0 * d1);
        wsum += e0 + e1;
        vsum += (e0 * b0 * d1 + e1 * b1 * d0) * r;
      }
    }
    if (abort_flag) break;
    const int gx = x0 + px, gy = y0 + py;
    if (gx < p.W && gy < p.H) {
      const float v = clampf(mean + 5.0f * vsum / wsum * stdv, 0.0f, 1.0f);
      if (XP) {
        stp2(out + (size_t)gy * p.out_pitch + 2 * gx, orig, v);
      } else {
        stp(out + (size_t)(2 * gy) * p.out_pitch + gx, orig);
        stp(out + (size_t)(2 * gy + 1) * p.out_pitch + gx, v);
      }
    }
    __syncthreads();  // A tile and tile free for the next tile
  }
  if (tid == 0) {  // no MMA may still write tensor memory when it is freed
    mma_commit(smem_u32(&mbar[2]));
    if (!mbar_wait_bounded(smem_u32(&mbar[2]), 0u)) abort_flag = 1;
  }
  __syncthreads();
  if (abort_flag && tid == 0) atomicCAS(p.err, 0, kErrWaitTimeout);
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TCOLS));
  }
}

template <int WH, int NNS, bool XP, typename T>
int launch_one(const NnArgs& a, cudaStream_t s) {
  constexpr int NT = 8 * WH;
  constexpr int DY0 = -(WH / 2 - 1);
  constexpr int TW = 32 + (XP ? WH / 2 - DY0 : 7), TH = 4 + (XP ? 7 : WH / 2 - DY0);
  // CTAs per SM are capped by tensor memory (512 columns per SM, 4*NC per
  // CTA): the shared-memory request is raised so that no more CTAs than fit
  // in TMEM can be resident, so tcgen05.alloc never waits on a neighbour.
  constexpr int NC = NNS < 32 ? NNS : 32;
  constexpr int per_sm = 512 / (4 * NC) > 4 ? 4 : 512 / (4 * NC);
  int dev = 0, sms = 0, sm_smem = 0, blk_smem = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return -95;
  cudaDeviceGetAttribute(&sm_smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  cudaDeviceGetAttribute(&blk_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  constexpr int KP = (NT + 3 + 15) / 16 * 16;
  const size_t need = (size_t)2 * NNS * KP * 2 + 128 * KP * 2 + TW * TH * 4;
  const size_t cap = (size_t)sm_smem / (per_sm + 1) + 1024;
  const size_t smem = need > cap ? need : cap;
  if (smem > (size_t)blk_smem) return -95;
  auto kern = nn_tc_kernel<WH, NNS, XP, T>;
  static bool configured[64] = {};  // per instantiation and device
  if (!configured[dev]) {
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
      return -5;
    configured[dev] = true;
  }
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int ntiles = ((a.W + 31) / 32) * ((a.H + 3) / 4);
  const int grid = ntiles < sms * per_sm ? ntiles : sms * per_sm;
  kern<<<grid, kThreads, smem, s>>>(a);
  return 0;
}

template <int WH, bool XP, typename T>
int dispatch_nns(const NnArgs& a, cudaStream_t s) {
  switch (a.nns) {
    case 16: return launch_one<WH, 16, XP, T>(a, s);
    case 32: return launch_one<WH, 32, XP, T>(a, s);
    case 64: return launch_one<WH, 64, XP, T>(a, s);
    case 128: return launch_one<WH, 128, XP, T>(a, s);
    case 256: return launch_one<WH, 256, XP, T>(a, s);
  }
  return -95;
}

template <typename T>
int launch_t(const NnArgs& a, bool xp, cudaStream_t s) {
  if (a.win_h == 4) return xp ? dispatch_nns<4, true, T>(a, s) : dispatch_nns<4, false, T>(a, s);
  if (a.win_h == 6) return xp ? dispatch_nns<6, true, T>(a, s) : dispatch_nns<6, false, T>(a, s);
  return -95;
}

}  // namespace

bool nnedi3_tc_supported(int nns, int win_h) {
  return (nns == 16 || nns == 32 || nns == 64 || nns == 128 || nns == 256) && (win_h == 4 || win_h == 6);
}

int nnedi3_tc_chunk(int nns) { return nns < 32 ? nns : 32; }

int launch_nnedi3_tc(const NnArgs& a, bool xpass, int dtype, cudaStream_t s) {
  if (!a.wts_h || !a.err) return -22;
  return dtype == 0 ? launch_t<float>(a, xpass, s) : launch_t<__half>(a, xpass, s);
}

}  // namespace pz
