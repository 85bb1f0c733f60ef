// NNEDI3 doubling pass on the 5th-generation tensor cores (tcgen05).
//
// Reference arithmetic: nnedi3-nns16-win8x4.hook:20-50 (normalise the 8xK
// window, nns neuron pairs, exp-weighted Elliott blend); pass geometry as in
// the CUDA-core kernel (nnedi3_simt.cu).
//
// One persistent CTA works through tiles of 128 interpolated pixels (32
// consecutive pixels x 4 rows) with two warp-specialised roles:
//
//   producers (warps 0-3, one thread per pixel): stage the window tile,
//     normalise each pixel's window, x_hat = (x - mean) * invstd, and write
//     it as one FP16 row of the A operand [128 x KP] (K-major, no-swizzle
//     core matrices) together with the row's mean / std / original sample;
//     thread 0 then issues the tile's tcgen05.mma.kind::f16 instructions
//     (M = 128, N = min(2 nns, 256)) against the resident weight operand B
//     and commits them to mbarriers.  A, the per-pixel values and the TMEM
//     accumulator are double-buffered, so tile i+1 is normalised and its
//     MMAs run while tile i is in the epilogue;
//   epilogue (2 warps per TMEM lane quarter): after the accumulator's
//     mbarrier, warp w reads lanes 32 (w % 4) .. +31 -- one lane per pixel --
//     of its half of the neuron columns with tcgen05.ld and runs the blend in
//     FP32 (e = exp2 of the softmax branch, already in log2 units; Elliott
//     b / (1 + |b|); wsum, vsum); the two halves meet in shared memory and
//     the first writes the pixel pair.
//
// Every wait is bounded (kWaitNs of %globaltimer): a wait that runs out
// marks the thread's state failed; the group barriers (bar.red.and) make
// that decision uniform per role, the CTA leaves its loop, waits (bounded)
// for its own MMAs to complete, frees its tensor memory and reports
// kErrWaitTimeout in the device error word.
#include "async.cuh"
#include "kernels.h"

namespace pz {
namespace {

constexpr int kEpiGroups = 2;                         // epilogue warps per TMEM lane quarter
constexpr int kThreads = 128 + 128 * kEpiGroups;      // producers + epilogue
constexpr int kProducerBar = 1, kEpilogueBar = 2;     // named barrier ids

// Neurons per TMEM read group: NC softmax columns followed by NC Elliott
// columns (the host stores B chunk-major in the same grouping).
__host__ __device__ constexpr int nn_chunk(int nns) { return nns / 2 < 32 ? nns / 2 : 32; }

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

// Arrive on `mbar` once every tcgen05 operation this thread issued so far
// has completed.
__device__ __forceinline__ void mma_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t mbar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(mbar) : "memory");
}

// Named barrier over `count` threads that also ANDs a predicate across them.
__device__ __forceinline__ bool bar_and(int id, int count, bool v) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.u32 p, %1, 0;\n\t"
      "bar.red.and.pred q, %2, %3, p;\n\t"
      "selp.u32 %0, 1, 0, q;\n\t}\n"
      : "=r"(r)
      : "r"((uint32_t)v), "r"(id), "r"(count)
      : "memory");
  return r != 0;
}

// N consecutive accumulator columns of this thread's TMEM lane.
template <int N>
__device__ __forceinline__ void tmem_ld(uint32_t taddr, float (&v)[N]) {
  uint32_t r[N];
  if constexpr (N == 32) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
  } else if constexpr (N == 16) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
  } else {
    static_assert(N == 8, "TMEM read width");
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
  }
#pragma unroll
  for (int i = 0; i < N; i++) v[i] = __uint_as_float(r[i]);
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

// mbarriers of the pipeline (index into the CTA's barrier array)
enum : int {
  kAccFull = 0,    // [2] MMAs of an accumulator buffer done        (tcgen05.commit)
  kAccEmpty = 2,   // [2] every epilogue warp has read that buffer   (4 * kEpiGroups arrivals)
  kAFree = 4,      // [2] the MMAs reading an A buffer are done      (tcgen05.commit)
  kPixFull = 6,    // [2] A rows and pixel values of a stage written (producer thread 0)
  kPixEmpty = 8,   // [2] the pixel values of a stage are read       (4 arrivals)
  kDrain = 10,     // all MMAs of the CTA are done                   (tcgen05.commit)
  kNumBars = 11
};

template <int NNS>
constexpr int ctas_per_sm() {
  // TMEM: two accumulator buffers of min(2 nns, 256) columns out of 512;
  // threads: at most 2048 per SM; at most 2 so the registers suffice
  constexpr int cols = 2 * (2 * NNS < 256 ? 2 * NNS : 256);
  return 512 / cols >= 2 ? 2 : 1;
}

template <int WH, int NNS, bool XP, typename T>
__global__ void __launch_bounds__(kThreads, ctas_per_sm<NNS>()) nn_tc_kernel(const __grid_constant__ NnArgs p) {
  constexpr int NT = 8 * WH;                     // window taps
  constexpr int KP = (NT + 3 + 15) / 16 * 16;    // K: taps, mean term, bias hi/lo, zero pad
  constexpr int NC = nn_chunk(NNS);              // neurons per TMEM read group
  constexpr int CB = 2 * NNS < 256 ? 2 * NNS : 256;  // accumulator columns per MMA chunk
  constexpr int NMC = 2 * NNS / CB;              // MMA chunks per tile
  constexpr int NCC = CB / (2 * NC);             // read groups per MMA chunk
  constexpr int NCG = NCC / kEpiGroups;          // ... per epilogue group
  constexpr int TCOLS = 2 * CB;                  // two accumulator buffers
  constexpr int DY0 = -(WH / 2 - 1);
  constexpr int OX0 = XP ? DY0 : -3, OX1 = XP ? WH / 2 : 4;
  constexpr int OY0 = XP ? -3 : DY0, OY1 = XP ? 4 : WH / 2;
  constexpr int TW = 32 + OX1 - OX0, TH = 4 + OY1 - OY0;
  constexpr uint32_t SBO = KP * 16;              // bytes between 8-row groups (A and B)
  constexpr uint32_t LBO = 128;                  // bytes between K-adjacent core matrices
  constexpr uint32_t ABYTES = 128 * KP * 2;      // one A buffer
  static_assert(NCC % kEpiGroups == 0 && NCG >= 1, "neuron groups must split evenly between epilogue warps");
  static_assert(TCOLS >= 32 && (TCOLS & (TCOLS - 1)) == 0, "TMEM allocation must be a power of two >= 32");

  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char* sB = smem;                                      // [2*NNS][KP] f16
  unsigned char* sA = sB + 2 * NNS * KP * 2;                     // [2][128][KP] f16
  float* tile = reinterpret_cast<float*>(sA + 2 * ABYTES);       // [TH][TW]
  float4* pix = reinterpret_cast<float4*>(tile + ((TW * TH + 3) & ~3));  // [2][128]: mean, std, original
  float2* red = reinterpret_cast<float2*>(pix + 2 * 128);        // [2][128]: second half's (wsum, vsum)
  __shared__ __align__(8) unsigned long long bars[kNumBars];
  __shared__ uint32_t tmem_base;

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
    for (int b = 0; b < 2; b++) {
      mbar_init(smem_u32(&bars[kAccFull + b]), 1);
      mbar_init(smem_u32(&bars[kAccEmpty + b]), 4 * kEpiGroups);
      mbar_init(smem_u32(&bars[kAFree + b]), 1);
      mbar_init(smem_u32(&bars[kPixFull + b]), 1);
      mbar_init(smem_u32(&bars[kPixEmpty + b]), 4);
    }
    mbar_init(smem_u32(&bars[kDrain]), 1);
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base;
  auto bar = [&](int i) { return smem_u32(&bars[i]); };

  const int tiles_x = (p.W + 31) / 32, tiles_y = (p.H + 3) / 4;
  const int ntiles = tiles_x * tiles_y;
  bool ok = true;

  if (warp < 4) {
    // ------------------------------------------------------- producers ---
    const T* in = static_cast<const T*>(p.in);
    const uint32_t a_addr = smem_u32(sA), b_addr = smem_u32(sB);
    constexpr uint32_t IDESC = instr_desc(128, CB);
    // the window tile of the next tile is loaded into registers while the
    // current tile is normalised (at most PF values per thread)
    constexpr int PF = (TW * TH + 127) / 128;
    float pre[PF];
    auto prefetch = [&](int t) {
      if (t >= ntiles) return;
      const int px0 = (t % tiles_x) * 32, py0 = (t / tiles_x) * 4;
#pragma unroll
      for (int r = 0; r < PF; r++) {
        const int i = tid + r * 128;
        if (i < TW * TH) {
          const int ty = i / TW, tx = i % TW;
          const int gx = clampi(px0 + OX0 + tx, 0, p.W - 1), gy = clampi(py0 + OY0 + ty, 0, p.H - 1);
          pre[r] = ldp(in + (size_t)gy * p.in_pitch + gx);
        }
      }
    };
    prefetch(blockIdx.x);
    int it = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, it++) {
      const int s = it & 1;
      if (it >= 2) {  // A[s] and pix[s] were last used by tile it-2
        const uint32_t par = ((it >> 1) - 1) & 1;
        ok = ok && mbar_wait_bounded(bar(kAFree + s), par);
        ok = ok && mbar_wait_bounded(bar(kPixEmpty + s), par);
      }
#pragma unroll
      for (int r = 0; r < PF; r++) {
        const int i = tid + r * 128;
        if (i < TW * TH) tile[i] = pre[r];
      }
      if (!bar_and(kProducerBar, 128, ok)) {
        ok = false;
        break;
      }
      prefetch(t + gridDim.x);  // in flight while this tile is normalised
      // ---- normalise this thread's window into its A row (pixel m = tid)
      const int m = tid, px = lane, py = warp;
      float xv[NT];
      float sum = 0.0f;
#pragma unroll
      for (int k = 0; k < NT; k++) {
        const int dx = k % 8 - 3, dy = k / 8 + DY0;
        const int ox = XP ? dy : dx, oy = XP ? dx : dy;
        xv[k] = tile[(py + oy - OY0) * TW + px + ox - OX0];
        sum += xv[k];
      }
      const float mean = sum / (float)NT;
      float var = 0.0f;
#pragma unroll
      for (int k = 0; k < NT; k++) {
        xv[k] -= mean;
        var += xv[k] * xv[k];
      }
      var /= (float)NT;
      const float invstd = var >= kFltEps ? rsqrtf(var) : 0.0f;
      {  // A row: [x_hat (NT), mean * invstd, 1, 1, 0...]
        unsigned char* row = sA + s * ABYTES + (m >> 3) * SBO + (m & 7) * 16;
        const float mterm = mean * invstd;
#pragma unroll
        for (int kc = 0; kc < KP / 8; kc++) {
          __half2 h[4];
#pragma unroll
          for (int j = 0; j < 4; j++) {
            const int k = 8 * kc + 2 * j;
            const float v0 = k < NT ? xv[k] * invstd : (k == NT ? mterm : (k <= NT + 2 ? 1.0f : 0.0f));
            const float v1 = k + 1 < NT ? xv[k + 1] * invstd
                                        : (k + 1 == NT ? mterm : (k + 1 <= NT + 2 ? 1.0f : 0.0f));
            h[j] = __floats2half2_rn(v0, v1);
          }
          *reinterpret_cast<uint4*>(row + kc * LBO) = *reinterpret_cast<uint4*>(h);
        }
      }
      pix[s * 128 + m] = make_float4(mean, var * invstd, tile[(py - OY0) * TW + px - OX0], 0.0f);
      fence_async_smem();  // the A rows are read by the tensor cores (async proxy)
      if (!bar_and(kProducerBar, 128, ok)) {
        ok = false;
        break;
      }
      if (tid == 0) {
        mbar_arrive(bar(kPixFull + s));
#pragma unroll 1
        for (int c = 0; c < NMC && ok; c++) {
          const int gc = it * NMC + c, b = gc & 1;
          if (gc >= 2) ok = mbar_wait_bounded(bar(kAccEmpty + b), ((gc >> 1) - 1) & 1);
          if (!ok) break;
          tc_fence_after();
#pragma unroll
          for (int ks = 0; ks < KP / 16; ks++) {
            const uint64_t ad = smem_desc(a_addr + s * ABYTES + ks * 2 * LBO, LBO, SBO);
            const uint64_t bd = smem_desc(b_addr + (uint32_t)c * (CB / 8) * SBO + ks * 2 * LBO, LBO, SBO);
            mma_f16(tmem + b * CB, ad, bd, IDESC, ks > 0 ? 1u : 0u);
          }
          mma_commit(bar(kAccFull + b));
        }
        if (ok) mma_commit(bar(kAFree + s));
      }
    }
  } else {
    // -------------------------------------------------------- epilogue ---
    const int q = warp & 3, g = (warp - 4) >> 2;   // TMEM lane quarter, neuron half
    const int m = 32 * q + lane;                   // pixel (TMEM lane) of this thread
    T* out = static_cast<T*>(p.out);
    const uint32_t lane_base = tmem + ((uint32_t)(32 * q) << 16);
    int it = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, it++) {
      const int s = it & 1;
      float4 pv = make_float4(0.f, 0.f, 0.f, 0.f);
      if (g == 0) {
        ok = ok && mbar_wait_bounded(bar(kPixFull + s), (it >> 1) & 1);
        pv = pix[s * 128 + m];
        __syncwarp();
        if (lane == 0) mbar_arrive(bar(kPixEmpty + s));
      }
      float wsum = 0.0f, vsum = 0.0f;
#pragma unroll 1
      for (int c = 0; c < NMC; c++) {
        const int gc = it * NMC + c, b = gc & 1;
        ok = ok && mbar_wait_bounded(bar(kAccFull + b), (gc >> 1) & 1);
        tc_fence_after();
#pragma unroll
        for (int k = 0; k < NCG; k++) {
          const uint32_t col = b * CB + (g * NCG + k) * 2 * NC;
          float s1[NC], s2[NC];
          tmem_ld<NC>(lane_base + col, s1);
          tmem_ld<NC>(lane_base + col + NC, s2);
          tmem_wait_ld();
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
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(bar(kAccEmpty + b));
      }
      if (g != 0) red[s * 128 + m] = make_float2(wsum, vsum);
      if (!bar_and(kEpilogueBar, 128 * kEpiGroups, ok)) {
        ok = false;
        break;
      }
      if (g == 0) {
#pragma unroll
        for (int h = 1; h < kEpiGroups; h++) {  // kEpiGroups == 2: one partner half
          const float2 o = red[s * 128 + m];
          wsum += o.x;
          vsum += o.y;
        }
        const int x0 = (t % tiles_x) * 32, y0 = (t / tiles_x) * 4;
        const int gx = x0 + lane, gy = y0 + q;
        if (gx < p.W && gy < p.H) {
          const float v = clampf(pv.x + 5.0f * vsum / wsum * pv.y, 0.0f, 1.0f);
          if (XP) {
            stp2(out + (size_t)gy * p.out_pitch + 2 * gx, pv.z, v);
          } else {
            stp(out + (size_t)(2 * gy) * p.out_pitch + gx, pv.z);
            stp(out + (size_t)(2 * gy + 1) * p.out_pitch + gx, v);
          }
        }
      }
    }
  }
  // ---- teardown: no MMA may still write tensor memory when it is freed
  if (tid == 0) {
    mma_commit(bar(kDrain));
    if (!mbar_wait_bounded(bar(kDrain), 0u)) ok = false;
  }
  tc_fence_before();
  const int all_ok = __syncthreads_and(ok);
  if (!all_ok && tid == 0) atomicCAS(p.err, 0, kErrWaitTimeout);
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TCOLS));
  }
}

template <int WH, int NNS, bool XP, typename T>
int launch_one(const NnArgs& a, cudaStream_t s) {
  constexpr int NT = 8 * WH;
  constexpr int KP = (NT + 3 + 15) / 16 * 16;
  constexpr int DY0 = -(WH / 2 - 1);
  constexpr int TW = 32 + (XP ? WH / 2 - DY0 : 7), TH = 4 + (XP ? 7 : WH / 2 - DY0);
  // CTAs per SM are capped (tensor memory, registers): the shared-memory
  // request is raised so that no more CTAs than that can be resident, so
  // tcgen05.alloc never waits on a neighbour.
  constexpr int per_sm = ctas_per_sm<NNS>();
  int dev = 0, sms = 0, sm_smem = 0, blk_smem = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return -95;
  cudaDeviceGetAttribute(&sm_smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  cudaDeviceGetAttribute(&blk_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const size_t need = (size_t)2 * NNS * KP * 2 + 2 * 128 * KP * 2 + (size_t)((TW * TH + 3) & ~3) * 4 +
                      2 * 128 * sizeof(float4) + 2 * 128 * sizeof(float2);
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

int nnedi3_tc_chunk(int nns) { return nn_chunk(nns); }

int launch_nnedi3_tc(const NnArgs& a, bool xpass, int dtype, cudaStream_t s) {
  if (!a.wts_h || !a.err) return -22;
  return dtype == 0 ? launch_t<float>(a, xpass, s) : launch_t<__half>(a, xpass, s);
}

}  // namespace pz
