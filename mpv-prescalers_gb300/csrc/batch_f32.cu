// Persistent batch kernel, float planes.
#include "batch_kernel.cuh"

namespace pz {

int launch_batch_f32(const DevJob* jobs, int n_jobs, int total, int* counter, int grid, cudaStream_t s) {
  batch_kernel<float><<<grid, kTileThreads, kBatchSmem, s>>>(jobs, n_jobs, total, counter);
  return 0;
}

int batch_fit_f32() {
  int fit = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, batch_kernel<float>, kTileThreads, kBatchSmem);
  return fit;
}

}  // namespace pz
