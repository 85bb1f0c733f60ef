// Asynchronous-copy helpers shared by the kernels: shared-memory addresses,
// bounded mbarrier waits and 2-D TMA tensor loads (sm_90+ PTX, used on sm_103a).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace pz {

constexpr unsigned long long kWaitNs = 1000000000ull;  // 1 s bound on every device-side wait

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count));
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t mbar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(mbar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Wait for phase `parity` of the mbarrier, giving up after `limit_ns`.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t mbar, uint32_t parity,
                                                  unsigned long long limit_ns = kWaitNs) {
  if (mbar_try(mbar, parity)) return true;
  const unsigned long long t0 = globaltimer();
  while (!mbar_try(mbar, parity)) {
    if (globaltimer() - t0 > limit_ns) return false;
  }
  return true;
}

// One arrival that also announces `bytes` of asynchronous copies.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
}

// 2-D tiled TMA load of the box at (x, y) of `map` into shared memory; the
// copy's bytes complete on `mbar`.  x * element size must be a multiple of
// 16 bytes; x and y may be negative or past the end (zero fill).
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
          "r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(mbar)
      : "memory");
}

}  // namespace pz
