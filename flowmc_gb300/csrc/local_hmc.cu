// local_hmc.cu -- instantiations of the K1 persistent local-step kernel for FMC_KERNEL_HMC
// (split per kernel kind so the instantiations compile in parallel).
#include "local_steps.cuh"

namespace fmc {
int launch_local_hmc(const LocalArgs& a, Shape sh, cudaStream_t st) {
  return launch_local_kind<FMC_KERNEL_HMC>(a, sh, st);
}
}  // namespace fmc
