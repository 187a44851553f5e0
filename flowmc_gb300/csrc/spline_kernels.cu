// spline_kernels.cu -- coupling-spline kernels: one warp per row, lanes over the
// transformed coordinates of the layer, log-determinants summed with a warp
// butterfly (deterministic order).
#include "flow.cuh"

namespace fmc {

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <int K, bool INV>
__global__ void __launch_bounds__(256) k_spline(const float* __restrict__ raw, float* __restrict__ xa,
                                                float* __restrict__ ld, int64_t n, int d, int nt, int tpar,
                                                SplineCfg cfg) {
  constexpr int P = 3 * K + 1;
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < n; r += warps) {
    const float* rr = raw + r * (int64_t)nt * P;
    float acc = 0.f;
    for (int t = lane; t < nt; t += 32) {
      float prm[P];
#pragma unroll
      for (int p = 0; p < P; ++p) prm[p] = __ldg(rr + t * P + p);
      Knots<K> kn;
      make_knots<K>(prm, cfg, kn);
      const int j = 2 * t + tpar;
      float* xp = xa + r * d + j;
      float out, l;
      if (INV) rqs_inv<K>(*xp, kn, out, l);
      else rqs_fwd<K>(*xp, kn, out, l);
      *xp = out;
      acc += l;
    }
    acc = warp_sum(acc);
    if (lane == 0) ld[r] += acc;
  }
}

template <int K>
__global__ void __launch_bounds__(256) k_spline_bwd(const float* __restrict__ raw, const float* __restrict__ xa,
                                                    const float* __restrict__ gy, float gld, float* __restrict__ graw,
                                                    float* __restrict__ gxa, int64_t n, int d, int nt, int tpar,
                                                    int cpar, SplineCfg cfg) {
  constexpr int P = 3 * K + 1;
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  const int ncond = d - nt;
  for (int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < n; r += warps) {
    const float* rr = raw + r * (int64_t)nt * P;
    float* gr = graw + r * (int64_t)nt * P;
    for (int t = lane; t < nt; t += 32) {
      float prm[P], g[P];
#pragma unroll
      for (int p = 0; p < P; ++p) prm[p] = __ldg(rr + t * P + p);
      Knots<K> kn;
      make_knots<K>(prm, cfg, kn);
      const int j = 2 * t + tpar;
      const float gx = rqs_fwd_adjoint<K>(xa[r * d + j], prm, cfg, kn, gy[r * d + j], gld, g);
      gxa[r * d + j] = gx;
#pragma unroll
      for (int p = 0; p < P; ++p) gr[t * P + p] = g[p];
    }
    for (int k = lane; k < ncond; k += 32) {
      const int j = 2 * k + cpar;
      gxa[r * d + j] = gy[r * d + j];
    }
  }
}

static int grid_for_rows(int64_t n) {
  int64_t b = (n + 7) / 8;
  const int64_t cap = (int64_t)sm_count() * 16;
  if (b > cap) b = cap;
  return (int)(b < 1 ? 1 : b);
}

#define FMC_FOR_BINS(X) X(2) X(3) X(4) X(5) X(6) X(8) X(10) X(12) X(16)

int launch_spline(int K, bool inverse, cudaStream_t st, const float* raw, float* xa, float* ld, int64_t n, int d,
                  int nt, int tpar, SplineCfg cfg) {
  if (n <= 0) return FMC_OK;
  const int grid = grid_for_rows(n);
#define CASE(k)                                                                              \
  if (K == k) {                                                                              \
    if (inverse) k_spline<k, true><<<grid, 256, 0, st>>>(raw, xa, ld, n, d, nt, tpar, cfg);  \
    else k_spline<k, false><<<grid, 256, 0, st>>>(raw, xa, ld, n, d, nt, tpar, cfg);         \
    FMC_LAUNCH_CHECK();                                                                      \
    return FMC_OK;                                                                           \
  }
  FMC_FOR_BINS(CASE)
#undef CASE
  set_error("n_bins=%d is not instantiated (2,3,4,5,6,8,10,12,16)", K);
  return FMC_ERR_UNSUPPORTED;
}

int launch_spline_bwd(int K, cudaStream_t st, const float* raw, const float* xa, const float* gy, float gld,
                      float* graw, float* gxa, int64_t n, int d, int nt, int tpar, int cpar, SplineCfg cfg) {
  if (n <= 0) return FMC_OK;
  const int grid = grid_for_rows(n);
#define CASE(k)                                                                                              \
  if (K == k) {                                                                                              \
    k_spline_bwd<k><<<grid, 256, 0, st>>>(raw, xa, gy, gld, graw, gxa, n, d, nt, tpar, cpar, cfg);           \
    FMC_LAUNCH_CHECK();                                                                                      \
    return FMC_OK;                                                                                           \
  }
  FMC_FOR_BINS(CASE)
#undef CASE
  set_error("n_bins=%d is not instantiated (2,3,4,5,6,8,10,12,16)", K);
  return FMC_ERR_UNSUPPORTED;
}

}  // namespace fmc
