// gemm_tc.cuh -- BF16 conditioner path (tcgen05/TMEM GEMMs fed by TMA, gemm_tc.cu).
#pragma once
#include <cuda_bf16.h>
#include "flow.cuh"

namespace fmc {

__device__ __forceinline__ uint16_t f32_to_bf16_rn(float v) {
  return __bfloat16_as_ushort(__float2bfloat16_rn(v));
}

// Conditioner MLP of layer l for rows [0, m) in BF16 with FP32 accumulation:
// cond (fp32 [m, n_c]) -> raw (fp32 [m, n_t*P]); cond16/h16a/h16b are bf16
// staging buffers with rows padded to 64 elements.
int conditioner_bf16(const FmcFlow* f, const FlowGeom& g, int l, int64_t m, const float* cond, uint16_t* cond16,
                     uint16_t* h16a, uint16_t* h16b, float* raw, cudaStream_t st);

size_t train_ws_bytes(const FlowGeom& g, int64_t n);

}  // namespace fmc
