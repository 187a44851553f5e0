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

// theta (fp32, packed) -> zero-padded bf16 weight segments (FlowGeom::w16_off)
int pack_bf16_weights(const FlowGeom& g, const float* theta, uint16_t* w16, cudaStream_t st);

// C = epi(A . B^T + bias) on tcgen05; A [M, lda] bf16 (K = lda valid columns,
// lda multiple of 64), B [rows_b >= N, ldb] bf16 (ldb == lda, rows_b multiple
// of 256), epi 0: tanh -> bf16 C [M, ldc] storing n_store columns (zeros
// beyond N); epi 1: + bias -> fp32 C [M, ldc] storing n_store (= N) columns.
int tc_gemm(cudaStream_t st, const uint16_t* A, int64_t M, int64_t rows_a, int K, const uint16_t* B, int N,
            int rows_b, const float* bias, void* C, int64_t ldc, int n_store, int epi);

}  // namespace fmc
