// flow.cuh -- geometry of the packed MaskedCouplingRQSpline parameters and the
// per-layer building blocks shared by the inference and training paths.
#pragma once
#include "common.cuh"
#include "spline.cuh"

namespace fmc {

struct FlowGeom {
  int d, L, nh, K, P;
  int H[FMC_MAX_HIDDEN];
  SplineCfg cfg;
  int64_t n_params;
  int64_t layer_off[FMC_MAX_LAYERS + 1];
  // padded bf16 copy of the Linear weights (BF16 path): segment l*(nh+1)+i is
  // W_i of layer l as [round_up(out, 256), round_up(in, 64)], zero padded
  int64_t w16_off[FMC_MAX_LAYERS * (FMC_MAX_HIDDEN + 1) + 1];
  // transposed copies W_i^T as [round_up(in, 256), w16t_cols] (training); the
  // last Linear's columns follow the padded d-raw layout (draw_cols)
  int64_t w16t_off[FMC_MAX_LAYERS * (FMC_MAX_HIDDEN + 1) + 1];
  // the last Linear of each layer re-packed in spline groups (fused inference
  // kernel, tc_spline.cu): group g = DG transformed coordinates x P rows,
  // padded to BN rows; [n_groups(l) * BN, round_up(H_last, 64)]
  int64_t w16g_off[FMC_MAX_LAYERS + 1];
  // spline groups: a coordinate's P raw parameters sit at a column pitch of
  // spl_pp = round_up(P, 8) (so the epilogue reads them with 8-column TMEM
  // loads at 8-aligned columns), spl_dg coordinates per group, spl_bn rows
  int spl_pp, spl_dg, spl_bn;
  // BF16 training: the spline adjoint writes d raw row-major with coordinate t
  // at columns [t * spl_opc, t * spl_opc + P) and zeros up to (t + 1) * spl_opc
  // (spl_opc = round_up(P, 8), so each coordinate is a whole number of 16-byte
  // chunks that one TMA box stores)
  int spl_opc;
  int wgrad_splits;   // FmcFlow::wgrad_splits (sizes the training workspace's split-K partials)
  int64_t n_w16;

  // conditioning coordinates of layer l: j = 2k + cpar(l); transformed: j = 2k + tpar(l)
  __host__ __device__ int cpar(int l) const { return 1 - (l & 1); }
  __host__ __device__ int tpar(int l) const { return l & 1; }
  __host__ __device__ int nc(int l) const { return (d - cpar(l) + 1) / 2; }
  __host__ __device__ int nt(int l) const { return d - nc(l); }
  int nc_max() const { return nc(0) > nc(1) ? nc(0) : nc(1); }
  int nt_max() const { return nt(0) > nt(1) ? nt(0) : nt(1); }
  int h_max() const {
    int m = 0;
    for (int i = 0; i < nh; ++i) m = H[i] > m ? H[i] : m;
    return m;
  }
  // linear layer i of layer l: in/out sizes and offsets (relative to layer_off[l])
  __host__ __device__ int lin_in(int l, int i) const { return i == 0 ? nc(l) : H[i - 1]; }
  __host__ __device__ int lin_out(int l, int i) const { return i == nh ? nt(l) * P : H[i]; }
  __host__ __device__ int64_t lin_w(int l, int i) const {
    int64_t o = 2;
    for (int u = 0; u < i; ++u) o += (int64_t)lin_out(l, u) * lin_in(l, u) + lin_out(l, u);
    return o;
  }
  int64_t lin_b(int l, int i) const { return lin_w(l, i) + (int64_t)lin_out(l, i) * lin_in(l, i); }
  __host__ __device__ static int64_t rup(int64_t v, int64_t a) { return (v + a - 1) / a * a; }
  __host__ __device__ int w16_rows(int l, int i) const { return (int)rup(lin_out(l, i), 256); }
  __host__ __device__ int w16_cols(int l, int i) const { return (int)rup(lin_in(l, i), 64); }
  __host__ __device__ int w16t_rows(int l, int i) const { return (int)rup(lin_in(l, i), 256); }
  __host__ __device__ int spl_groups(int l) const { return (nt(l) + spl_dg - 1) / spl_dg; }
  __host__ __device__ int64_t draw_cols(int l) const { return (int64_t)nt(l) * spl_opc; }
  __host__ __device__ int w16t_cols(int l, int i) const {
    return (int)rup(i == nh ? draw_cols(l) : (int64_t)lin_out(l, i), 64);
  }
};

int make_geom(const FmcFlow* f, FlowGeom& g);

// ScalarAffine of a coupling layer (common.py:229, 238): forward (v + t) e^s,
// inverse v e^-s - t, with es = e^(+-s); rounded explicitly so that every
// kernel applying it (k_affine, the fused spline kernel's next-layer fold)
// gives the same bits
__device__ __forceinline__ float scalar_affine(float v, float es, float t, int inverse) {
  return inverse ? __fmaf_rn(v, es, -t) : __fmul_rn(__fadd_rn(v, t), es);
}
// its log-determinant, d * (+-s)
__device__ __forceinline__ float scalar_affine_logdet(float s, int d, int inverse) {
  return __fmul_rn((float)d, inverse ? -s : s);
}

// --------------------------------------------------------------- kernels
__global__ void k_standardize(const float* __restrict__ x, int64_t n, int d, const float* __restrict__ aux,
                              float* __restrict__ out);
__global__ void k_destandardize(float* __restrict__ x, int64_t n, int d, const float* __restrict__ aux);
__global__ void k_affine(const float* __restrict__ in, float* __restrict__ out, float* __restrict__ cond,
                         uint16_t* __restrict__ cond16, int ldc16, int64_t n, int d, int nc, int cpar,
                         const float* __restrict__ th_layer, int inverse, float* __restrict__ ld, int ld_init);
__global__ void k_base_logprob(const float* __restrict__ y, const float* __restrict__ ld, int64_t n, int d,
                               const float* __restrict__ aux, float* __restrict__ logp);
__global__ void k_base_sample(const float* __restrict__ z, Rng rng, int64_t n, int d,
                              const float* __restrict__ aux, float* __restrict__ out);

// spline kernels, one warp per row; instantiated for the supported bin counts
int launch_spline(int K, bool inverse, cudaStream_t st, const float* raw, float* xa, float* ld, int64_t n, int d,
                  int nt, int tpar, SplineCfg cfg);
int launch_spline_bwd(int K, cudaStream_t st, const float* raw, const float* xa, const float* gy, float gld,
                      float* graw, float* gxa, int64_t n, int d, int nt, int tpar, int cpar, SplineCfg cfg);

}  // namespace fmc
