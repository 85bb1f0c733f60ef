// NNEDI3 doubling pass on the tcgen05 tensor cores (FP16 operands, FP32
// accumulation in tensor memory).  Placeholder until the kernel lands.
#include "kernels.h"

namespace pz {

bool nnedi3_tc_supported(int nns, int win_h) {
  (void)nns;
  (void)win_h;
  return false;
}

int launch_nnedi3_tc(const NnArgs& a, bool xpass, int dtype, cudaStream_t s) {
  (void)a;
  (void)xpass;
  (void)dtype;
  (void)s;
  return -95;
}

}  // namespace pz
