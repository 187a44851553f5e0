// gemm_tc.cu -- BF16 conditioner GEMMs on the 5th-generation tensor cores.
#include "gemm_tc.cuh"

namespace fmc {

int conditioner_bf16(const FmcFlow* f, const FlowGeom& g, int l, int64_t m, const float* cond, uint16_t* cond16,
                     uint16_t* h16a, uint16_t* h16b, float* raw, cudaStream_t st) {
  set_error("BF16 conditioner path not available in this build");
  return FMC_ERR_UNSUPPORTED;
}

}  // namespace fmc
