// gemm_simt.cuh -- FP32 SIMT GEMM with fused epilogues (the FP32 conditioner
// path; the BF16 path runs on tcgen05, gemm_tc.cu).
//
//   C[i, j] = beta * C[i, j] + sum_k A(i, k) * B(j, k)   (+ bias[j], tanh, ...)
//   A(i, k) = A[i*lda + k] (A_KMAJOR) or A[k*lda + i]
//   B(j, k) = B[j*ldb + k] (B_KMAJOR) or B[k*ldb + j]
//
// 64x64 output tile per 256-thread block, 4x4 per thread, K step 16, tiles
// staged through shared memory with bounds-predicated loads.
#pragma once
#include "common.cuh"

namespace fmc {

enum GemmEpi : int {
  EPI_NONE = 0,       // C = beta*C + AB
  EPI_BIAS = 1,       // C = AB + bias
  EPI_BIAS_TANH = 2,  // C = tanh(AB + bias)
  EPI_DTANH = 3,      // C = AB * (1 - aux^2)   (aux = tanh output of the forward)
  EPI_BIAS_RELU = 4,  // C = max(AB + bias, 0)
  EPI_DRELU = 5,      // C = AB where aux > 0, else 0   (aux = relu output of the forward)
};

template <bool A_KMAJOR, bool B_KMAJOR, int EPI>
__global__ void __launch_bounds__(256) k_sgemm(int M, int N, int K, const float* __restrict__ A, int64_t lda,
                                               const float* __restrict__ B, int64_t ldb,
                                               const float* __restrict__ bias, const float* __restrict__ aux,
                                               int64_t ldaux, float* __restrict__ C, int64_t ldc, float beta) {
  constexpr int BM = 64, BN = 64, BK = 16;
  __shared__ __align__(16) float As[BK][BM + 4];
  __shared__ __align__(16) float Bs[BK][BN + 4];
  const int tid = threadIdx.x;
  const int tx = tid % 16, ty = tid / 16;
  const int64_t i0 = (int64_t)blockIdx.y * BM, j0 = (int64_t)blockIdx.x * BN;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += BK) {
    // A tile: 64 x 16
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int e = tid + r * 256;
      int ii, kk;
      if (A_KMAJOR) { ii = e / BK; kk = e % BK; } else { kk = e / BM; ii = e % BM; }
      const int64_t gi = i0 + ii;
      const int gk = k0 + kk;
      float v = 0.f;
      if (gi < M && gk < K) v = A_KMAJOR ? A[gi * lda + gk] : A[(int64_t)gk * lda + gi];
      As[kk][ii] = v;
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int e = tid + r * 256;
      int jj, kk;
      if (B_KMAJOR) { jj = e / BK; kk = e % BK; } else { kk = e / BN; jj = e % BN; }
      const int64_t gj = j0 + jj;
      const int gk = k0 + kk;
      float v = 0.f;
      if (gj < N && gk < K) v = B_KMAJOR ? B[gj * ldb + gk] : B[(int64_t)gk * ldb + gj];
      Bs[kk][jj] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      const float4 a = *reinterpret_cast<const float4*>(&As[kk][ty * 4]);
      const float4 b = *reinterpret_cast<const float4*>(&Bs[kk][tx * 4]);
      const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int w = 0; w < 4; ++w) acc[u][w] = fmaf(av[u], bv[w], acc[u][w]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int64_t gi = i0 + ty * 4 + u;
    if (gi >= M) continue;
#pragma unroll
    for (int w = 0; w < 4; ++w) {
      const int64_t gj = j0 + tx * 4 + w;
      if (gj >= N) continue;
      float v = acc[u][w];
      float* cp = C + gi * ldc + gj;
      if (EPI == EPI_NONE) {
        if (beta != 0.f) v += beta * *cp;
      } else if (EPI == EPI_BIAS) {
        v += bias[gj];
      } else if (EPI == EPI_BIAS_TANH) {
        v = tanhf(v + bias[gj]);
      } else if (EPI == EPI_BIAS_RELU) {
        v = fmaxf(v + bias[gj], 0.f);
      } else if (EPI == EPI_DRELU) {
        v = (aux[gi * ldaux + gj] > 0.f) ? v : 0.f;
      } else {
        const float h = aux[gi * ldaux + gj];
        v = v * (1.f - h * h);
      }
      *cp = v;
    }
  }
}

template <bool A_KMAJOR, bool B_KMAJOR, int EPI>
inline int sgemm(cudaStream_t st, int64_t M, int N, int K, const float* A, int64_t lda, const float* B, int64_t ldb,
                 const float* bias, const float* aux, int64_t ldaux, float* C, int64_t ldc, float beta) {
  if (M <= 0 || N <= 0) return FMC_OK;
  dim3 grid((unsigned)((N + 63) / 64), (unsigned)((M + 63) / 64));
  if (grid.y > 65535u) {
    // split very tall problems
    const int64_t rows = 65535ll * 64;
    for (int64_t m0 = 0; m0 < M; m0 += rows) {
      const int64_t mm = (M - m0 < rows) ? (M - m0) : rows;
      const float* Ap = A_KMAJOR ? A + m0 * lda : A + m0;
      const float* auxp = aux ? aux + m0 * ldaux : nullptr;
      int rc = sgemm<A_KMAJOR, B_KMAJOR, EPI>(st, mm, N, K, Ap, lda, B, ldb, bias, auxp, ldaux, C + m0 * ldc, ldc, beta);
      if (rc) return rc;
    }
    return FMC_OK;
  }
  k_sgemm<A_KMAJOR, B_KMAJOR, EPI><<<grid, 256, 0, st>>>((int)M, N, K, A, lda, B, ldb, bias, aux, ldaux, C, ldc, beta);
  FMC_LAUNCH_CHECK();
  return FMC_OK;
}

// ------------------------------------------------------------------ split-K A^T B
// Weight gradients: out [M, N] = sum over K rows of A[k, :M]^T B[k, :N] with K
// (the batch) far larger than M and N, where one tile per output block would
// leave most SMs idle. The rows are cut into S slices, each slice's 64 x 64
// tile sums go to part[S][M][N], and k_sum_slices adds the slices in a fixed
// order (bitwise reproducible).
constexpr int kKouterMaxSlices = 64;

// part[z][i][j] = sum over rows k of slice z of A[k*lda + i] * B[k*ldb + j]
// (ONES: B = 1, N = 1 -- column sums). 64 x 64 tiles, 16 rows per step.
template <bool ONES>
__global__ void __launch_bounds__(256) k_sgemm_kouter(int M, int N, int64_t K, int64_t kslice,
                                                      const float* __restrict__ A, int64_t lda,
                                                      const float* __restrict__ B, int64_t ldb,
                                                      float* __restrict__ part) {
  constexpr int BM = 64, BN = 64, BK = 16;
  __shared__ __align__(16) float As[BK][BM + 4];
  __shared__ __align__(16) float Bs[BK][BN + 4];
  const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
  const int i0 = blockIdx.y * BM, j0 = blockIdx.x * BN;
  const int64_t kb = (int64_t)blockIdx.z * kslice;
  const int64_t ke = (kb + kslice < K) ? kb + kslice : K;
  float acc[4][4] = {};
  for (int64_t k0 = kb; k0 < ke; k0 += BK) {
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int e = tid + r * 256;
      const int kk = e / BM, ii = e % BM;
      const int64_t gk = k0 + kk;
      As[kk][ii] = (gk < ke && i0 + ii < M) ? A[gk * lda + i0 + ii] : 0.f;
      float b = 0.f;
      if (gk < ke && j0 + ii < N) b = ONES ? 1.f : B[gk * ldb + j0 + ii];
      Bs[kk][ii] = b;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      const float4 a = *reinterpret_cast<const float4*>(&As[kk][ty * 4]);
      const float4 b = *reinterpret_cast<const float4*>(&Bs[kk][tx * 4]);
      const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int w = 0; w < 4; ++w) acc[u][w] = fmaf(av[u], bv[w], acc[u][w]);
    }
    __syncthreads();
  }
  float* out = part + (int64_t)blockIdx.z * M * N;
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int gi = i0 + ty * 4 + u;
    if (gi >= M) continue;
#pragma unroll
    for (int w = 0; w < 4; ++w) {
      const int gj = j0 + tx * 4 + w;
      if (gj < N) out[(int64_t)gi * N + gj] = acc[u][w];
    }
  }
}

template <int U = 0>
__global__ void k_sum_slices(const float* __restrict__ part, int S, int64_t mn, float* __restrict__ out) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < mn; e += (int64_t)gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int z = 0; z < S; ++z) s += part[(int64_t)z * mn + e];
    out[e] = s;
  }
}

// out [M, N] = A^T B over K rows (A [K, lda], B [K, ldb]); ones: column sums
// of A. part holds part_floats floats of slice partials; with room for fewer
// than two slices the single slice is written to out directly.
inline int kouter(cudaStream_t st, int M, int N, int64_t K, const float* A, int64_t lda, const float* B, int64_t ldb,
                  bool ones, float* part, int64_t part_floats, float* out) {
  if (M <= 0 || N <= 0) return FMC_OK;
  const int64_t mn = (int64_t)M * N;
  const int64_t tiles = (int64_t)((N + 63) / 64) * ((M + 63) / 64);
  int64_t S = (2 * (int64_t)sm_count() + tiles - 1) / tiles;
  const int64_t by_rows = (K + 255) / 256;   // at least 256 rows per slice
  if (S > by_rows) S = by_rows;
  if (S > kKouterMaxSlices) S = kKouterMaxSlices;
  if (part == nullptr || S * mn > part_floats) S = part != nullptr ? part_floats / mn : 1;
  if (S < 1) S = 1;
  const int64_t kslice = (((K + S - 1) / S) + 15) / 16 * 16;
  S = (K + kslice - 1) / kslice;
  if (S < 1) S = 1;
  float* dst = S > 1 ? part : out;
  dim3 grid((unsigned)((N + 63) / 64), (unsigned)((M + 63) / 64), (unsigned)S);
  if (ones)
    k_sgemm_kouter<true><<<grid, 256, 0, st>>>(M, N, K, kslice, A, lda, nullptr, 0, dst);
  else
    k_sgemm_kouter<false><<<grid, 256, 0, st>>>(M, N, K, kslice, A, lda, B, ldb, dst);
  FMC_LAUNCH_CHECK();
  if (S > 1) {
    int64_t b = (mn + 255) / 256;
    const int64_t cap = (int64_t)sm_count() * 8;
    if (b > cap) b = cap;
    k_sum_slices<<<(unsigned)(b < 1 ? 1 : b), 256, 0, st>>>(part, (int)S, mn, out);
    FMC_LAUNCH_CHECK();
  }
  return FMC_OK;
}

}  // namespace fmc
