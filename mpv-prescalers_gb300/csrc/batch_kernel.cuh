// Persistent batch kernel over a table of RAVU tile jobs (see batch.cu).
// Instantiated once per plane dtype in batch_f32.cu / batch_f16.cu so the two
// large kernels compile in parallel.
#pragma once
#include "ravu_tiles.cuh"

namespace pz {

// Tile programs a batch can run (program id = index).
enum Prog : int {
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

struct DevJob {
  RavuArgs a;
  int prog;
  int tiles_w;
  int first_tile;  // prefix sum within its launch group
  int pad;
};

// H: the program set of the kernel -- false: programs 0..44 (FP32 LUT
// texels, and the ravu lattice in every form); true: 45..71 (the fast form's
// FP16-texel lite / 3x / zoom programs).  Two kernels per plane dtype keep
// each translation unit's instantiations (and compile time) bounded.
template <typename T, bool H>
__device__ __forceinline__ void run_prog(int prog, const RavuArgs& a, int x0, int y0, float* smem) {
#define PZ_CASE(id, ...) \
  case id: __VA_ARGS__::run(a, x0, y0, smem); return;
  if constexpr (!H) {
  switch (prog) {
    PZ_CASE(0, LiteTile<2, false, T>) PZ_CASE(1, LiteTile<2, true, T>)
    PZ_CASE(2, LiteTile<3, false, T>) PZ_CASE(3, LiteTile<3, true, T>)
    PZ_CASE(4, LiteTile<4, false, T>) PZ_CASE(5, LiteTile<4, true, T>)
    PZ_CASE(6, ThreeXTile<2, kLuma, T>) PZ_CASE(7, ThreeXTile<2, kYuv, T>) PZ_CASE(8, ThreeXTile<2, kRgb, T>)
    PZ_CASE(9, ThreeXTile<3, kLuma, T>) PZ_CASE(10, ThreeXTile<3, kYuv, T>) PZ_CASE(11, ThreeXTile<3, kRgb, T>)
    PZ_CASE(12, ThreeXTile<4, kLuma, T>) PZ_CASE(13, ThreeXTile<4, kYuv, T>) PZ_CASE(14, ThreeXTile<4, kRgb, T>)
    PZ_CASE(15, Int11Tile<2, kLuma, T>) PZ_CASE(16, Int11Tile<2, kYuv, T>) PZ_CASE(17, Int11Tile<2, kRgb, T>)
    PZ_CASE(18, Int11Tile<3, kLuma, T>) PZ_CASE(19, Int11Tile<3, kYuv, T>) PZ_CASE(20, Int11Tile<3, kRgb, T>)
    PZ_CASE(21, Int11Tile<4, kLuma, T>) PZ_CASE(22, Int11Tile<4, kYuv, T>) PZ_CASE(23, Int11Tile<4, kRgb, T>)
    PZ_CASE(24, LatticeTile<2, kLuma, T>) PZ_CASE(25, LatticeTile<2, kYuv, T>) PZ_CASE(26, LatticeTile<2, kRgb, T>)
    PZ_CASE(27, LatticeTile<3, kLuma, T>) PZ_CASE(28, LatticeTile<3, kYuv, T>) PZ_CASE(29, LatticeTile<3, kRgb, T>)
    PZ_CASE(30, LatticeTile<4, kLuma, T>) PZ_CASE(31, LatticeTile<4, kYuv, T>) PZ_CASE(32, LatticeTile<4, kRgb, T>)
    PZ_CASE(33, ZoomTile<2, kLuma, false, T>) PZ_CASE(34, ZoomTile<2, kLuma, true, T>)
    PZ_CASE(35, ZoomTile<2, kYuv, false, T>) PZ_CASE(36, ZoomTile<2, kYuv, true, T>)
    PZ_CASE(37, ZoomTile<2, kRgb, false, T>) PZ_CASE(38, ZoomTile<2, kRgb, true, T>)
    PZ_CASE(39, ZoomTile<3, kLuma, false, T>) PZ_CASE(40, ZoomTile<3, kLuma, true, T>)
    PZ_CASE(41, ZoomTile<3, kYuv, false, T>) PZ_CASE(42, ZoomTile<3, kYuv, true, T>)
    PZ_CASE(43, ZoomTile<3, kRgb, false, T>) PZ_CASE(44, ZoomTile<3, kRgb, true, T>)
  }
  } else {
  switch (prog) {
    PZ_CASE(45, LiteTile<2, false, T, true>) PZ_CASE(46, LiteTile<2, true, T, true>)
    PZ_CASE(47, LiteTile<3, false, T, true>) PZ_CASE(48, LiteTile<3, true, T, true>)
    PZ_CASE(49, LiteTile<4, false, T, true>) PZ_CASE(50, LiteTile<4, true, T, true>)
    PZ_CASE(51, ThreeXTile<2, kLuma, T, true>) PZ_CASE(52, ThreeXTile<2, kYuv, T, true>)
    PZ_CASE(53, ThreeXTile<2, kRgb, T, true>) PZ_CASE(54, ThreeXTile<3, kLuma, T, true>)
    PZ_CASE(55, ThreeXTile<3, kYuv, T, true>) PZ_CASE(56, ThreeXTile<3, kRgb, T, true>)
    PZ_CASE(57, ThreeXTile<4, kLuma, T, true>) PZ_CASE(58, ThreeXTile<4, kYuv, T, true>)
    PZ_CASE(59, ThreeXTile<4, kRgb, T, true>)
    PZ_CASE(60, ZoomTile<2, kLuma, false, T, true>) PZ_CASE(61, ZoomTile<2, kLuma, true, T, true>)
    PZ_CASE(62, ZoomTile<2, kYuv, false, T, true>) PZ_CASE(63, ZoomTile<2, kYuv, true, T, true>)
    PZ_CASE(64, ZoomTile<2, kRgb, false, T, true>) PZ_CASE(65, ZoomTile<2, kRgb, true, T, true>)
    PZ_CASE(66, ZoomTile<3, kLuma, false, T, true>) PZ_CASE(67, ZoomTile<3, kLuma, true, T, true>)
    PZ_CASE(68, ZoomTile<3, kYuv, false, T, true>) PZ_CASE(69, ZoomTile<3, kYuv, true, T, true>)
    PZ_CASE(70, ZoomTile<3, kRgb, false, T, true>) PZ_CASE(71, ZoomTile<3, kRgb, true, T, true>)
  }
  }
#undef PZ_CASE
}

constexpr size_t cmax(size_t a, size_t b) { return a > b ? a : b; }
// Largest tile program (lattice r4 rgb, zoom r3 rgb, lite r4 ar).
constexpr size_t kBatchSmem = cmax(cmax(LatticeTile<4, kRgb, float>::smem_bytes, ZoomTile<3, kRgb, true, float>::smem_bytes),
                                   cmax(LiteTile<4, true, float>::smem_bytes, ThreeXTile<4, kRgb, float>::smem_bytes));

// Persistent CTAs: claim tile numbers from `counter` until `total` is reached.
template <typename T, bool H>
__global__ void __launch_bounds__(kTileThreads) batch_kernel(const DevJob* __restrict__ jobs, int n_jobs, int total,
                                                             int* counter) {
  extern __shared__ float4 bsmem[];
  __shared__ RavuArgs s_args;
  __shared__ int s_item, s_job, s_prog, s_tw, s_first;
  float* smem = reinterpret_cast<float*>(bsmem);
  for (;;) {
    if (threadIdx.x == 0) {
      const int item = atomicAdd(counter, 1);
      s_item = item;
      if (item < total) {  // last job whose first tile <= item
        int lo = 0, hi = n_jobs - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (jobs[mid].first_tile <= item) lo = mid; else hi = mid - 1;
        }
        s_job = lo;
        s_prog = jobs[lo].prog;
        s_tw = jobs[lo].tiles_w;
        s_first = jobs[lo].first_tile;
      }
    }
    __syncthreads();
    const int item = s_item;
    if (item >= total) break;
    {  // job arguments into shared memory (broadcast reads in the tile program)
      const int* src = reinterpret_cast<const int*>(&jobs[s_job].a);
      int* dst = reinterpret_cast<int*>(&s_args);
      for (int i = threadIdx.x; i < (int)(sizeof(RavuArgs) / 4); i += kTileThreads) dst[i] = src[i];
    }
    __syncthreads();
    const int t = item - s_first;
    run_prog<T, H>(s_prog, s_args, (t % s_tw) * kTileW, (t / s_tw) * kTileH, smem);
    __syncthreads();  // the tile's shared memory is free for the next claim
  }
}


// One persistent launch of the kernel for plane dtype `dt` (PZ_F32 / PZ_F16)
// and program set `h`; batch_fit: its resident CTAs per SM.
#define PZ_BATCH_DECL(sfx)                                                                          \
  int launch_batch_##sfx(const DevJob* jobs, int n_jobs, int total, int* counter, int grid, cudaStream_t s); \
  int batch_fit_##sfx();
PZ_BATCH_DECL(f32)
PZ_BATCH_DECL(f16)
PZ_BATCH_DECL(f32h)
PZ_BATCH_DECL(f16h)
#undef PZ_BATCH_DECL

// Instantiation of one (dtype, program set) kernel in its own translation unit.
#define PZ_BATCH_DEFINE(sfx, T, H)                                                                  \
  int launch_batch_##sfx(const DevJob* jobs, int n_jobs, int total, int* counter, int grid, cudaStream_t s) { \
    batch_kernel<T, H><<<grid, kTileThreads, kBatchSmem, s>>>(jobs, n_jobs, total, counter);        \
    return 0;                                                                                       \
  }                                                                                                 \
  int batch_fit_##sfx() {                                                                           \
    int fit = 0;                                                                                    \
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, batch_kernel<T, H>, kTileThreads, kBatchSmem); \
    return fit;                                                                                     \
  }

}  // namespace pz
