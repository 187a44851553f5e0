// flow_train.cu -- K6: loss and hand-written gradient of MaskedCouplingRQSpline
// maximum-likelihood training (NFModel.loss_fn / train_step,
// nf_model/base.py:98-125).
//
// Forward: the standardised batch runs through the layers; only each layer's
// INPUT is kept ([L+1, n, d] floats). Backward, layer by layer in reverse:
// the ScalarAffine output, the conditioning block and the conditioner's tanh
// activations and outputs are recomputed from the saved input, then
//   spline adjoint (spline.cuh)        -> d raw params, d x (transformed)
//   conditioner adjoint (GEMMs)        -> d W, d b, d cond
//   ScalarAffine adjoint               -> d x (layer input), d scale, d shift
// All reductions (bias columns, scale/shift, loss) are two-stage with a fixed
// order, so gradients are bitwise reproducible.
#include "flow.cuh"
#include "gemm_simt.cuh"
#include "gemm_tc.cuh"

namespace fmc {

static int64_t a256(int64_t v) { return (v + 255) / 256 * 256; }

struct TrainWs {
  float *xs, *xa, *cond, *hs, *raw, *graw, *gh0, *gh1, *gcond, *gy, *gxa, *ld, *logp, *part;
  int64_t part_floats;
  // FP32 path: split-K partials of the weight-gradient GEMMs (K = the batch)
  float* spart;
  int64_t spart_floats;
  // fused last-Linear + spline kernels (BF16 path): log-det partials and
  // per-128-row-tile bias-gradient partials; split-K partials of the
  // weight-gradient GEMMs (K = the batch)
  float *ldp, *bpart, *kpart, *colpart;
  int64_t kpart_floats;
  // BF16 path (tensor-core GEMMs): activations and gradients, row-major (the
  // weight-gradient GEMMs read them MN-major, so no transposed copies)
  uint16_t *cond16, *hs16, *graw16, *gz16[2];
  int64_t n128, n64, hld, ncld, pld;
};

static int colsum_blocks(int64_t n) {
  int64_t rb = (n + 511) / 512;
  if (rb > 128) rb = 128;
  return (int)(rb < 1 ? 1 : rb);
}

static void carve_train(const FlowGeom& g, int64_t n, bool bf16, void* ws, TrainWs& w, size_t* total) {
  char* p = (char*)ws;
  int64_t used = 0;
  auto take = [&](int64_t floats) {
    float* r = (float*)(p + used);
    used += a256(4 * floats);
    return r;
  };
  auto take16 = [&](int64_t elems) {
    uint16_t* r = (uint16_t*)(p + used);
    used += a256(2 * elems);
    return r;
  };
  const int64_t ntP = (int64_t)g.nt_max() * g.P;
  w.xs = take((int64_t)(g.L + 1) * n * g.d);
  w.xa = take(n * g.d);
  w.cond = take(n * g.nc_max());
  // fp32 conditioner activations and gradients: the FP32 path only
  w.hs = bf16 ? nullptr : take((int64_t)g.nh * n * g.h_max());
  w.raw = bf16 ? nullptr : take(n * ntP);
  w.graw = bf16 ? nullptr : take(n * ntP);
  w.gh0 = bf16 ? nullptr : take(n * g.h_max());
  w.gh1 = bf16 ? nullptr : take(n * g.h_max());
  w.gcond = take(n * g.nc_max());
  w.gy = take(n * g.d);
  w.gxa = take(n * g.d);
  w.ld = take(n);
  w.logp = take(n);
  int64_t m = ntP > g.h_max() ? ntP : g.h_max();
  if (m < 4096) m = 4096;
  w.part_floats = (int64_t)colsum_blocks(n) * m;
  w.part = take(w.part_floats);
  w.spart = nullptr;
  w.spart_floats = 0;
  if (!bf16) {
    int64_t mn = 1;
    for (int l = 0; l < g.L; ++l)
      for (int i = 0; i <= g.nh; ++i) {
        const int64_t f = (int64_t)g.lin_out(l, i) * g.lin_in(l, i);
        if (f > mn) mn = f;
      }
    int64_t s = (int64_t)(16 << 20) / mn;   // about 64 MB of partials at most
    if (s > kKouterMaxSlices) s = kKouterMaxSlices;
    if (s < 2) s = 2;
    w.spart_floats = s * mn;
    w.spart = take(w.spart_floats);
  }
  w.ldp = w.bpart = w.kpart = w.colpart = nullptr;
  w.kpart_floats = 0;
  w.cond16 = w.hs16 = w.graw16 = nullptr;
  w.gz16[0] = w.gz16[1] = nullptr;
  if (bf16) {
    w.n128 = FlowGeom::rup(n, 128);
    w.n64 = FlowGeom::rup(n, 64);
    w.hld = FlowGeom::rup(g.h_max(), 64);
    w.ncld = FlowGeom::rup(g.nc_max(), 64);
    w.pld = FlowGeom::rup((int64_t)g.nt_max() * g.spl_opc, 64);   // padded d-raw rows
    w.cond16 = take16(w.n128 * w.ncld);
    w.hs16 = take16((int64_t)g.nh * w.n128 * w.hld);
    w.graw16 = take16(w.n128 * w.pld);
    for (int k = 0; k < 2; ++k) {
      w.gz16[k] = take16(w.n128 * w.hld);
    }
    const int64_t groups = (g.nt_max() + g.spl_dg - 1) / g.spl_dg;
    w.ldp = take(n * kSplineEpiPerQuarter * groups);
    w.bpart = take((w.n128 / 128) * kSplineBwdRowParts * ntP);
    for (int l = 0; l < g.L; ++l)
      for (int i = 0; i <= g.nh; ++i) {
        // the last Linear's weight gradient runs over the padded d-raw rows
        const int64_t mrows = i == g.nh ? g.draw_cols(l) : g.lin_out(l, i);
        const int64_t f = (int64_t)splitk_scratch_floats(mrows, g.lin_in(l, i), (int)w.n64, g.wgrad_splits);
        if (f > w.kpart_floats) w.kpart_floats = f;
      }
    w.kpart = w.kpart_floats > 0 ? take(w.kpart_floats) : nullptr;
    // per-32-row column sums of the tanh-adjoint GEMM outputs (hidden bias gradients)
    w.colpart = take((w.n128 / 32) * g.h_max());
  }
  if (total) *total = (size_t)used;
}

size_t train_ws_bytes(const FlowGeom& g, int64_t n, bool bf16) {
  TrainWs w;
  size_t tot = 0;
  carve_train(g, n, bf16, nullptr, w, &tot);
  return tot;
}

// ------------------------------------------------------------------ kernels
__global__ void k_colsum_partial(const float* __restrict__ gm, int64_t n, int m, int64_t rows_per,
                                 float* __restrict__ part) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= m) return;
  const int64_t r0 = blockIdx.y * rows_per;
  int64_t r1 = r0 + rows_per;
  if (r1 > n) r1 = n;
  float s = 0.f;
  for (int64_t r = r0; r < r1; ++r) s += gm[r * m + j];
  part[(int64_t)blockIdx.y * m + j] = s;
}

__global__ void k_colsum_final(const float* __restrict__ part, int rb, int m, float* __restrict__ out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= m) return;
  float s = 0.f;
  for (int b = 0; b < rb; ++b) s += part[(int64_t)b * m + j];
  out[j] = s;
}

// out[j] = sum over rows of part[r * m + j] for a tall partial matrix: a
// block takes 32 columns, its 32 warps rows w, w + 32, ... (coalesced
// 128-byte loads), then the 32 per-warp sums are added in warp order
__global__ void __launch_bounds__(1024) k_colsum_rows(const float* __restrict__ part, int rows, int m,
                                                      float* __restrict__ out) {
  __shared__ float sh[32][33];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int j = blockIdx.x * 32 + lane;
  float s = 0.f;
  if (j < m)
#pragma unroll 4
    for (int r = w; r < rows; r += 32) s += part[(int64_t)r * m + j];
  sh[w][lane] = s;
  __syncthreads();
  if (w == 0 && j < m) {
    float t = 0.f;
#pragma unroll
    for (int k = 0; k < 32; ++k) t += sh[k][lane];
    out[j] = t;
  }
}

static int colsum(cudaStream_t st, const float* gm, int64_t n, int m, float* part, float* out) {
  const int rb = colsum_blocks(n);
  const int64_t rows_per = (n + rb - 1) / rb;
  dim3 grid((m + 255) / 256, rb);
  k_colsum_partial<<<grid, 256, 0, st>>>(gm, n, m, rows_per, part);
  FMC_LAUNCH_CHECK();
  k_colsum_final<<<(m + 255) / 256, 256, 0, st>>>(part, rb, m, out);
  FMC_LAUNCH_CHECK();
  return FMC_OK;
}

__global__ void k_colsum_partial_bf16(const uint16_t* __restrict__ gm, int64_t n, int m, int64_t ld,
                                      int64_t rows_per, float* __restrict__ part) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= m) return;
  const int64_t r0 = blockIdx.y * rows_per;
  int64_t r1 = r0 + rows_per;
  if (r1 > n) r1 = n;
  float s = 0.f;
  for (int64_t r = r0; r < r1; ++r) s += __uint_as_float((uint32_t)gm[r * ld + j] << 16);
  part[(int64_t)blockIdx.y * m + j] = s;
}

static int colsum_bf16(cudaStream_t st, const uint16_t* gm, int64_t n, int m, int64_t ld, float* part, float* out) {
  const int rb = colsum_blocks(n);
  const int64_t rows_per = (n + rb - 1) / rb;
  dim3 grid((m + 255) / 256, rb);
  k_colsum_partial_bf16<<<grid, 256, 0, st>>>(gm, n, m, ld, rows_per, part);
  FMC_LAUNCH_CHECK();
  k_colsum_final<<<(m + 255) / 256, 256, 0, st>>>(part, rb, m, out);
  FMC_LAUNCH_CHECK();
  return FMC_OK;
}

template <int NT>
__device__ __forceinline__ float block_sum(float v, float* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  float r = 0.f;
  if (threadIdx.x < 32) {
    r = (lane < NT / 32) ? sh[lane] : 0.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
  }
  return r;  // valid in thread 0
}

// loss = -mean(logp): one block, fixed order
__global__ void __launch_bounds__(1024) k_loss(const float* __restrict__ logp, int64_t n, float* __restrict__ loss) {
  __shared__ float sh[32];
  float s = 0.f;
  for (int64_t i = threadIdx.x; i < n; i += 1024) s += logp[i];
  s = block_sum<1024>(s, sh);
  if (threadIdx.x == 0) *loss = -s / (float)n;
}

// gradient of the loss at the flow output: d/dy (-logN(y; 0, cI))/n = y / (c n)
__global__ void k_init_gy(const float* __restrict__ y, int64_t tot, int d, const float* __restrict__ aux, float inv_n,
                          float* __restrict__ gy) {
  const float c = aux[2 * d];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < tot; i += (int64_t)gridDim.x * blockDim.x)
    gy[i] = y[i] / c * inv_n;
}

// adjoint of xa = (x + t) e^s and of the conditioning gather;
// writes d x and per-block partial sums of d t and (sum gxa * xa). One warp
// per row (lanes over the coordinates), rows strided over the grid.
__global__ void __launch_bounds__(256) k_affine_bwd(const float* __restrict__ gxa, const float* __restrict__ gcond,
                                                    const float* __restrict__ xa, int64_t n, int d, int nc, int cpar,
                                                    const float* __restrict__ th_layer, float* __restrict__ gx,
                                                    float* __restrict__ part) {
  __shared__ float sh[32];
  const float es = expf(th_layer[0]);
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  float st = 0.f, ss = 0.f;
  for (int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < n; r += warps) {
    const float* gr = gxa + r * d;
    const float* xr = xa + r * d;
    const float* cr = gcond + r * nc;
    float* out = gx + r * d;
    for (int j = lane; j < d; j += 32) {
      float g = gr[j];
      if ((j & 1) == cpar) g += cr[j >> 1];
      const float gv = g * es;
      out[j] = gv;
      st += gv;
      ss += g * xr[j];
    }
  }
  st = block_sum<256>(st, sh);
  ss = block_sum<256>(ss, sh);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = st;
    part[2 * blockIdx.x + 1] = ss;
  }
}

// the ScalarAffine's two gradients from the nb block partials: one warp,
// lane i summing partials i, i + 32, ..., then a fixed-order butterfly
__global__ void k_affine_param_grad(const float* __restrict__ part, int nb, float ld_term, float* __restrict__ g_layer) {
  const int lane = threadIdx.x & 31;
  float st = 0.f, ss = 0.f;
  for (int b = lane; b < nb; b += 32) {
    st += part[2 * b];
    ss += part[2 * b + 1];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    st += __shfl_xor_sync(0xffffffffu, st, o);
    ss += __shfl_xor_sync(0xffffffffu, ss, o);
  }
  if (threadIdx.x == 0) {
    g_layer[0] = ss + ld_term;  // d/d scale
    g_layer[1] = st;            // d/d shift
  }
}

static int ew_blocks(int64_t tot) {
  int64_t b = (tot + 255) / 256;
  const int64_t cap = (int64_t)sm_count() * 8;
  if (b > cap) b = cap;
  return (int)(b < 1 ? 1 : b);
}

// recompute layer l's conditioner on cond: hidden tanh activations into hs, output into raw
static int recompute_mlp(const FmcFlow* f, const FlowGeom& g, int l, int64_t n, TrainWs& w, cudaStream_t st) {
  const float* th = f->theta + g.layer_off[l];
  const float* a = w.cond;
  int in = g.nc(l);
  for (int i = 0; i <= g.nh; ++i) {
    const int out = g.lin_out(l, i);
    float* c = (i == g.nh) ? w.raw : w.hs + (int64_t)i * n * g.h_max();
    int rc = (i == g.nh)
                 ? sgemm<true, true, EPI_BIAS>(st, n, out, in, a, in, th + g.lin_w(l, i), in, th + g.lin_b(l, i), nullptr, 0, c, out, 0.f)
                 : sgemm<true, true, EPI_BIAS_TANH>(st, n, out, in, a, in, th + g.lin_w(l, i), in, th + g.lin_b(l, i), nullptr, 0, c, out, 0.f);
    if (rc) return rc;
    a = c;
    in = out;
  }
  return FMC_OK;
}

// BF16 recompute of layer l's conditioner hidden layers (from the bf16
// conditioning block k_affine left in w.cond16): tanh activations in bf16;
// the last Linear is recomputed inside the fused spline adjoint
static int recompute_hidden_bf16(const FmcFlow* f, const FlowGeom& g, int l, int64_t n, TrainWs& w, cudaStream_t st) {
  const float* th = f->theta + g.layer_off[l];
  int rc = FMC_OK;
  const uint16_t* a = w.cond16;
  for (int i = 0; i < g.nh; ++i) {
    const int seg = l * (g.nh + 1) + i;
    const int K = g.w16_cols(l, i), N = g.lin_out(l, i);
    tc::EpiArgs ep{};
    ep.bias = th + g.lin_b(l, i);
    uint16_t* h = w.hs16 + (int64_t)i * w.n128 * w.hld;
    const int ldo = (int)FlowGeom::rup(N, 64);
    if ((rc = tc_gemm(st, a, n, w.n128, K, f->theta_bf16 + g.w16_off[seg], N, g.w16_rows(l, i), ep, h, ldo, ldo,
                      tc::TC_EPI_TANH_BF16, f->gemm_bn, f->tile_rows == 256, 0, f->gemm_stages)))
      return rc;
    a = h;
  }
  return FMC_OK;
}

// BF16 adjoint of the conditioner: d raw (w.graw16, bf16, with the last bias
// gradient already reduced) -> weight/bias gradients into gl, d cond into
// w.gcond. The weight gradients read the row-major gradients and activations
// MN-major (tc_gemm_wgrad); rows [n, 64) of every operand are zero when n < 64.
static int backward_mlp_bf16(const FmcFlow* f, const FlowGeom& g, int l, int64_t n, TrainWs& w, float* gl,
                             cudaStream_t st) {
  int rc = FMC_OK;
  const uint16_t* gcur = w.graw16;
  int64_t ldcur = w.pld;
  int nxt = 0;
  bool have_cp = false;   // w.colpart holds the column sums of gcur
  for (int i = g.nh; i >= 0; --i) {
    const int out = g.lin_out(l, i), in = g.lin_in(l, i);
    const int seg = l * (g.nh + 1) + i;
    const uint16_t* act = (i == 0) ? w.cond16 : w.hs16 + (int64_t)(i - 1) * w.n128 * w.hld;
    const int64_t ldact = FlowGeom::rup(in, 64);
    // the last Linear's d raw is in the padded layout (coordinate t at columns
    // [t * opc, t * opc + P)): its weight gradient runs over the padded rows
    // and maps them back to t * P + p; its input-gradient GEMM contracts the
    // padded columns against the matching padded W^T
    const bool padded = i == g.nh;
    const int gcols = padded ? (int)g.draw_cols(l) : out;
    // dW = g^T a  [out, in], reduced over the batch (split along it when the
    // [out, in] tile grid is small)
    tc::EpiArgs e0{};
    e0.kpart = w.kpart;
    e0.kpart_floats = w.kpart_floats;
    e0.kslices = f->wgrad_splits;
    if (padded) {
      e0.rmap_grp = g.spl_opc;
      e0.rmap_keep = g.P;
    }
    if ((rc = tc_gemm_wgrad(st, gcur, ldcur, gcols, act, ldact, in, n, e0, gl + g.lin_w(l, i), in))) return rc;
    const int kg = padded ? g.w16t_cols(l, i) : (int)FlowGeom::rup(out, 64);
    if (padded && g.draw_cols(l) < kg) {
      // columns [draw_cols, kg) of d raw: zeros (a layer with fewer
      // transformed coordinates than the buffer's widest leaves older values)
      FMC_CUDA_TRY(cudaMemset2DAsync(w.graw16 + g.draw_cols(l), (size_t)w.pld * 2, 0,
                                     (size_t)(kg - g.draw_cols(l)) * 2, (size_t)n, st));
    }
    if (i < g.nh) {
      if (have_cp) {
        // fixed-order reduction of the per-32-row partials the DTANH GEMM left
        k_colsum_rows<<<(out + 31) / 32, 1024, 0, st>>>(w.colpart, (int)(w.n128 / 32), out, gl + g.lin_b(l, i));
        FMC_LAUNCH_CHECK();
      } else if ((rc = colsum_bf16(st, gcur, n, out, FlowGeom::rup(out, 64), w.part, gl + g.lin_b(l, i)))) {
        return rc;
      }
    }
    const uint16_t* WT = f->theta_bf16 + g.w16t_off[seg];
    if (i > 0) {
      // d a = (g W) * (1 - a^2), a = the tanh activation feeding Linear i
      tc::EpiArgs e1{};
      e1.aux = w.hs16 + (int64_t)(i - 1) * w.n128 * w.hld;
      e1.ldaux = FlowGeom::rup(in, 64);
      const int ldo = (int)FlowGeom::rup(in, 64);
      have_cp = tc_gemm_stages_output(w.gz16[nxt], ldo, ldo, n);
      if (have_cp) {
        e1.colpart = w.colpart;
        e1.ldpart = in;
      }
      if ((rc = tc_gemm(st, gcur, n, w.n128, kg, WT, in, g.w16t_rows(l, i), e1, w.gz16[nxt], ldo, ldo,
                        tc::TC_EPI_DTANH_BF16, 0, false, ldcur)))
        return rc;
      gcur = w.gz16[nxt];
      ldcur = ldo;
      nxt ^= 1;
    } else {
      tc::EpiArgs e2{};
      if ((rc = tc_gemm(st, gcur, n, w.n128, kg, WT, in, g.w16t_rows(l, i), e2, w.gcond, in, in, tc::TC_EPI_F32, 0,
                        false, ldcur)))
        return rc;
    }
  }
  return FMC_OK;
}

int flow_loss_grad(const FmcFlow* f, const float* x, int64_t n, float* loss, float* grad, void* ws, size_t ws_bytes,
                   cudaStream_t st) {
  FlowGeom g;
  int rc = make_geom(f, g);
  if (rc) return rc;
  FMC_CHECK_ARG(f->theta && f->aux, "flow theta/aux is NULL");
  FMC_CHECK_ARG(n >= 1, "n=%lld < 1", (long long)n);
  FMC_CHECK_ARG(x && loss && grad, "NULL array");
  const bool bf16 = f->precision == FMC_PREC_BF16;
  const size_t need = train_ws_bytes(g, n, bf16);
  FMC_CHECK_ARG(ws && ws_bytes >= need, "workspace of %zu bytes < %zu needed", ws_bytes, need);
  FMC_CHECK_ARG(((uintptr_t)ws & 255) == 0, "workspace must be 256-byte aligned");
  if (bf16) FMC_CHECK_ARG(f->theta_bf16 != nullptr, "BF16 mode needs theta_bf16");
  TrainWs w;
  carve_train(g, n, bf16, ws, w, nullptr);
  const int d = g.d;
  const int64_t nd = n * d;
  const int eb = ew_blocks(nd);
  int rb;   // one warp per row
  {
    int64_t b = (n + 7) / 8;
    if (b > (int64_t)sm_count() * 16) b = (int64_t)sm_count() * 16;
    rb = (int)(b < 1 ? 1 : b);
  }

  // ---- forward, saving layer inputs
  k_standardize<<<eb, 256, 0, st>>>(x, n, d, f->aux, w.xs);
  FMC_LAUNCH_CHECK();
  for (int l = 0; l < g.L; ++l) {
    float* xin = w.xs + (int64_t)l * nd;
    float* xout = w.xs + (int64_t)(l + 1) * nd;
    k_affine<<<rb, 256, 0, st>>>(xin, xout, bf16 ? nullptr : w.cond, bf16 ? w.cond16 : nullptr, g.w16_cols(l, 0),
                                 n, d, g.nc(l), g.cpar(l), f->theta + g.layer_off[l], 0, w.ld, l == 0 ? 1 : 0);
    FMC_LAUNCH_CHECK();
    if (bf16) {
      // the inference path: hidden layers, then the last Linear fused with the spline
      const uint16_t* h_last = nullptr;
      if ((rc = conditioner_bf16_hidden(f, g, l, n, nullptr, w.cond16, w.gz16[0], w.gz16[1], &h_last, st))) return rc;
      if ((rc = tc_linear_spline(st, g, f, l, h_last, n, w.n128, false, xout, w.ld, w.ldp))) return rc;
    } else {
      if ((rc = recompute_mlp(f, g, l, n, w, st))) return rc;
      if ((rc = launch_spline(g.K, false, st, w.raw, xout, w.ld, n, d, g.nt(l), g.tpar(l), g.cfg))) return rc;
    }
  }
  const float* y = w.xs + (int64_t)g.L * nd;
  {
    int64_t blocks = (n + 7) / 8;
    if (blocks > (int64_t)sm_count() * 16) blocks = (int64_t)sm_count() * 16;
    k_base_logprob<<<(int)blocks, 256, 0, st>>>(y, w.ld, n, d, f->aux, w.logp);
    FMC_LAUNCH_CHECK();
  }
  k_loss<<<1, 1024, 0, st>>>(w.logp, n, loss);
  FMC_LAUNCH_CHECK();

  // ---- backward
  const float inv_n = 1.0f / (float)n;
  const float gld = -inv_n;
  if (bf16 && n < 64) {
    // the weight-gradient GEMMs read 64-row blocks of the bf16 operands: rows
    // [n, 64) stay zero (the kernels below write rows < n only)
    FMC_CUDA_TRY(cudaMemsetAsync(w.cond16, 0, (size_t)64 * w.ncld * 2, st));
    for (int i = 0; i < g.nh; ++i)
      FMC_CUDA_TRY(cudaMemsetAsync(w.hs16 + (int64_t)i * w.n128 * w.hld, 0, (size_t)64 * w.hld * 2, st));
    FMC_CUDA_TRY(cudaMemsetAsync(w.graw16, 0, (size_t)64 * w.pld * 2, st));
    for (int k = 0; k < 2; ++k) FMC_CUDA_TRY(cudaMemsetAsync(w.gz16[k], 0, (size_t)64 * w.hld * 2, st));
  }
  k_init_gy<<<eb, 256, 0, st>>>(y, nd, d, f->aux, inv_n, w.gy);
  FMC_LAUNCH_CHECK();
  for (int l = g.L - 1; l >= 0; --l) {
    const float* th = f->theta + g.layer_off[l];
    float* gl = grad + g.layer_off[l];
    const float* xin = w.xs + (int64_t)l * nd;
    // the layer's spline input, and its conditioning block as the first
    // GEMM's operand (bf16, zero padded) or in fp32
    k_affine<<<rb, 256, 0, st>>>(xin, w.xa, bf16 ? nullptr : w.cond, bf16 ? w.cond16 : nullptr,
                                 bf16 ? g.w16_cols(l, 0) : 0, n, d, g.nc(l), g.cpar(l), th, 0, nullptr, 0);
    FMC_LAUNCH_CHECK();
    if (bf16) {
      // hidden activations, then the last Linear recomputed inside the fused
      // spline adjoint, which leaves d raw in the padded bf16 layout
      if ((rc = recompute_hidden_bf16(f, g, l, n, w, st))) return rc;
      const uint16_t* h_last = g.nh > 0 ? w.hs16 + (int64_t)(g.nh - 1) * w.n128 * w.hld : w.cond16;
      if ((rc = tc_linear_spline_bwd(st, g, f, l, h_last, n, w.n128, w.xa, w.gy, gld, w.gxa, w.graw16, w.pld,
                                     w.bpart)))
        return rc;
      const int ntP = g.lin_out(l, g.nh);
      k_colsum_rows<<<(ntP + 31) / 32, 1024, 0, st>>>(w.bpart, (int)(w.n128 / 128) * kSplineBwdRowParts, ntP,
                                                    gl + g.lin_b(l, g.nh));
      FMC_LAUNCH_CHECK();
      if ((rc = backward_mlp_bf16(f, g, l, n, w, gl, st))) return rc;
    } else {
      if ((rc = recompute_mlp(f, g, l, n, w, st))) return rc;
      if ((rc = launch_spline_bwd(g.K, st, w.raw, w.xa, w.gy, gld, w.graw, w.gxa, n, d, g.nt(l), g.tpar(l), g.cpar(l),
                                  g.cfg)))
        return rc;
      // conditioner adjoint
      const float* gcur = w.graw;
      float* gbufs[2] = {w.gh0, w.gh1};
      for (int i = g.nh; i >= 0; --i) {
        const int out = g.lin_out(l, i), in = g.lin_in(l, i);
        const float* a_in = (i == 0) ? w.cond : w.hs + (int64_t)(i - 1) * n * g.h_max();
        // dW = g^T a_in  [out, in], split along the batch
        if ((rc = kouter(st, out, in, n, gcur, out, a_in, in, false, w.spart, w.spart_floats, gl + g.lin_w(l, i))))
          return rc;
        if ((rc = colsum(st, gcur, n, out, w.part, gl + g.lin_b(l, i)))) return rc;
        float* gnext = (i == 0) ? w.gcond : gbufs[i & 1];
        if (i > 0) {
          if ((rc = sgemm<true, false, EPI_DTANH>(st, n, in, out, gcur, out, th + g.lin_w(l, i), in, nullptr, a_in,
                                                  in, gnext, in, 0.f)))
            return rc;
        } else {
          if ((rc = sgemm<true, false, EPI_NONE>(st, n, in, out, gcur, out, th + g.lin_w(l, i), in, nullptr,
                                                 nullptr, 0, gnext, in, 0.f)))
            return rc;
        }
        gcur = gnext;
      }
    }
    // ScalarAffine adjoint -> d(layer input) into gy
    const int ab = eb < 1024 ? eb : 1024;
    k_affine_bwd<<<ab, 256, 0, st>>>(w.gxa, w.gcond, w.xa, n, d, g.nc(l), g.cpar(l), th, w.gy, w.part);
    FMC_LAUNCH_CHECK();
    k_affine_param_grad<<<1, 32, 0, st>>>(w.part, ab, gld * (float)d * (float)n, gl);
    FMC_LAUNCH_CHECK();
  }
  return FMC_OK;
}

}  // namespace fmc

extern "C" int fmc_flow_loss_grad(const FmcFlow* flow, const float* x, int64_t n, float* loss, float* grad, void* ws,
                                  size_t ws_bytes, void* stream) {
  return fmc::flow_loss_grad(flow, x, n, loss, grad, ws, ws_bytes, (cudaStream_t)stream);
}
