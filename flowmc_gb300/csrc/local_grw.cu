// local_grw.cu -- instantiations of the K1 persistent local-step kernel for FMC_KERNEL_GRW
// (split per kernel kind so the instantiations compile in parallel).
#include "local_steps.cuh"

namespace fmc {
int launch_local_grw(const LocalArgs& a, Shape sh, cudaStream_t st) {
  return launch_local_kind<FMC_KERNEL_GRW>(a, sh, st);
}
}  // namespace fmc
