// flow.cu -- MaskedCouplingRQSpline inference: layout, forward, inverse,
// log_prob and sample entry points (K3/K4).
//
// Per layer l (rqSpline.py:450-488, common.py:127-168, 211-240):
//   k_affine        ScalarAffine (x + t) e^s (or its inverse) and the gather of
//                   the conditioning coordinates into a dense [n, n_c] block
//   conditioner     Linear+tanh ... Linear on the packed weights
//                   (FP32: SIMT GEMMs with fused bias/tanh epilogues;
//                    BF16: tcgen05 GEMMs, gemm_tc.cu)
//   k_spline        RQ spline (or inverse) of the transformed coordinates,
//                   log-determinants summed per row
// Rows are processed in chunks sized to keep the conditioner outputs
// (n_t * (3K+1) floats per row) within a bounded workspace.
#include "flow.cuh"
#include "gemm_simt.cuh"
#include "gemm_tc.cuh"

namespace fmc {

int make_geom(const FmcFlow* f, FlowGeom& g) {
  FMC_CHECK_ARG(f != nullptr, "flow is NULL");
  FMC_CHECK_ARG(f->n_dim >= 2 && f->n_dim <= 4096, "flow n_dim=%d outside [2, 4096]", f->n_dim);
  FMC_CHECK_ARG(f->n_layers >= 1 && f->n_layers <= FMC_MAX_LAYERS, "n_layers=%d outside [1, %d]", f->n_layers,
                FMC_MAX_LAYERS);
  FMC_CHECK_ARG(f->n_hidden >= 1 && f->n_hidden <= FMC_MAX_HIDDEN, "n_hidden=%d outside [1, %d]", f->n_hidden,
                FMC_MAX_HIDDEN);
  FMC_CHECK_ARG(f->n_bins >= 2 && f->n_bins <= 16, "n_bins=%d outside [2, 16]", f->n_bins);
  FMC_CHECK_ARG(f->range_max > f->range_min, "empty spline range");
  FMC_CHECK_ARG(f->gemm_stages == 0 || f->gemm_stages == 3 || f->gemm_stages == 4, "gemm_stages=%d not 0, 3 or 4",
                f->gemm_stages);
  FMC_CHECK_ARG(f->wgrad_splits >= 0 && f->wgrad_splits <= 32, "wgrad_splits=%d outside [0, 32]", f->wgrad_splits);
  FMC_CHECK_ARG(f->min_bin_size > 0.f && f->min_bin_size * f->n_bins < f->range_max - f->range_min,
                "min_bin_size incompatible with the range");
  g.d = f->n_dim;
  g.L = f->n_layers;
  g.nh = f->n_hidden;
  g.K = f->n_bins;
  g.P = 3 * f->n_bins + 1;
  for (int i = 0; i < FMC_MAX_HIDDEN; ++i) g.H[i] = i < g.nh ? f->hidden[i] : 0;
  for (int i = 0; i < g.nh; ++i) FMC_CHECK_ARG(g.H[i] >= 1 && g.H[i] <= 8192, "hidden[%d]=%d invalid", i, g.H[i]);
  g.cfg.rmin = f->range_min;
  g.cfg.rmax = f->range_max;
  g.cfg.min_bin = f->min_bin_size;
  g.cfg.min_slope = f->min_knot_slope;
  // rqSpline.py:37-38, in float32 as the reference's parameter dtype
  g.cfg.slope_offset = logf(expf(1.0f - f->min_knot_slope) - 1.0f);
  int64_t off = 0;
  for (int l = 0; l < g.L; ++l) {
    g.layer_off[l] = off;
    off += g.lin_b(l, g.nh) + g.lin_out(l, g.nh);
  }
  g.layer_off[g.L] = off;
  g.n_params = off;
  int64_t o16 = 0;
  for (int l = 0; l < g.L; ++l)
    for (int i = 0; i <= g.nh; ++i) {
      g.w16_off[l * (g.nh + 1) + i] = o16;
      o16 += (int64_t)g.w16_rows(l, i) * g.w16_cols(l, i);
    }
  g.w16_off[g.L * (g.nh + 1)] = o16;
  g.spl_pp = (g.P + 7) / 8 * 8;
  g.spl_dg = 256 / g.spl_pp;
  g.spl_bn = ((g.spl_dg * g.spl_pp + 15) / 16) * 16;
  g.spl_opc = g.spl_pp;
  g.wgrad_splits = f->wgrad_splits;
  for (int l = 0; l < g.L; ++l)
    for (int i = 0; i <= g.nh; ++i) {
      g.w16t_off[l * (g.nh + 1) + i] = o16;
      o16 += (int64_t)g.w16t_rows(l, i) * g.w16t_cols(l, i);
    }
  g.w16t_off[g.L * (g.nh + 1)] = o16;
  for (int l = 0; l < g.L; ++l) {
    g.w16g_off[l] = o16;
    o16 += (int64_t)g.spl_groups(l) * g.spl_bn * g.w16_cols(l, g.nh);
  }
  g.w16g_off[g.L] = o16;
  g.n_w16 = o16;
  return FMC_OK;
}

// ------------------------------------------------------------------ kernels
// one warp per row (lanes over the coordinates, rows strided over the grid):
// no per-element index division
__global__ void k_standardize(const float* __restrict__ x, int64_t n, int d, const float* __restrict__ aux,
                              float* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < n; r += warps)
    for (int j = lane; j < d; j += 32) out[r * d + j] = (x[r * d + j] - aux[j]) / sqrtf(aux[d + j]);
}

__global__ void k_destandardize(float* __restrict__ x, int64_t n, int d, const float* __restrict__ aux) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < n; r += warps)
    for (int j = lane; j < d; j += 32) x[r * d + j] = x[r * d + j] * sqrtf(aux[d + j]) + aux[j];
}

// one warp per row: ScalarAffine of every coordinate, the conditioning
// coordinates gathered into cond (fp32 [n, nc]) and/or cond16 (bf16 [n, ldc16],
// columns nc..ldc16 zeroed: the operand of the first tensor-core GEMM)
__global__ void k_affine(const float* __restrict__ in, float* __restrict__ out, float* __restrict__ cond,
                         uint16_t* __restrict__ cond16, int ldc16, int64_t n, int d, int nc, int cpar,
                         const float* __restrict__ th_layer, int inverse, float* __restrict__ ld, int ld_init) {
  const float s = th_layer[0], t = th_layer[1];
  const float es = expf(inverse ? -s : s);
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  // four coordinates per lane when every row is 16-byte aligned and the
  // conditioning coordinates (every other one) are exactly half of them
  const bool v4 = (d % 4 == 0) && 2 * nc == d && ((uintptr_t)in & 15) == 0 && ((uintptr_t)out & 15) == 0 &&
                  (cond == nullptr || ((uintptr_t)cond & 7) == 0) &&
                  (cond16 == nullptr || (((uintptr_t)cond16 & 3) == 0 && (ldc16 & 1) == 0));
  // one float4 of row r (coordinates 4q .. 4q + 3): out, and the two
  // conditioning ones among them (4q + cpar, 4q + 2 + cpar = conditioning 2q, 2q + 1)
  auto put4 = [&](int64_t r, int q, float4 a) {
    float4 o;
    o.x = scalar_affine(a.x, es, t, inverse);
    o.y = scalar_affine(a.y, es, t, inverse);
    o.z = scalar_affine(a.z, es, t, inverse);
    o.w = scalar_affine(a.w, es, t, inverse);
    reinterpret_cast<float4*>(out + r * d)[q] = o;
    const float c0 = cpar ? o.y : o.x, c1 = cpar ? o.w : o.z;
    if (cond != nullptr) reinterpret_cast<float2*>(cond + r * nc)[q] = make_float2(c0, c1);
    if (cond16 != nullptr)
      reinterpret_cast<uint32_t*>(cond16 + r * ldc16)[q] =
          (uint32_t)f32_to_bf16_rn(c0) | ((uint32_t)f32_to_bf16_rn(c1) << 16);
  };
  auto row_tail = [&](int64_t r) {
    if (cond16 != nullptr)
      for (int c = nc + lane; c < ldc16; c += 32) cond16[r * ldc16 + c] = 0;
    if (ld != nullptr && lane == 0) {
      const float l = scalar_affine_logdet(s, d, inverse);
      ld[r] = ld_init ? l : __fadd_rn(ld[r], l);
    }
  };
  const int64_t first = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (v4 && d <= 128) {
    // a row is at most one float4 per lane: two rows per iteration, both
    // loads issued before either is used (more bytes in flight per warp)
    const int q = lane;
    const bool lane_on = q < d / 4;
    for (int64_t r = first; r < n; r += 2 * warps) {
      const int64_t r1 = r + warps;
      const bool has1 = r1 < n;
      float4 a0 = make_float4(0.f, 0.f, 0.f, 0.f), a1 = a0;
      if (lane_on) {
        a0 = reinterpret_cast<const float4*>(in + r * d)[q];
        if (has1) a1 = reinterpret_cast<const float4*>(in + r1 * d)[q];
      }
      if (lane_on) put4(r, q, a0);
      row_tail(r);
      if (has1) {
        if (lane_on) put4(r1, q, a1);
        row_tail(r1);
      }
    }
    return;
  }
  for (int64_t r = first; r < n; r += warps) {
    const float* ir = in + r * d;
    float* orow = out + r * d;
    if (v4) {
      for (int q = lane; q < d / 4; q += 32) put4(r, q, reinterpret_cast<const float4*>(ir)[q]);
    } else {
      for (int j = lane; j < d; j += 32) {
        const float v = scalar_affine(ir[j], es, t, inverse);
        orow[j] = v;
        if ((j & 1) == cpar) {
          if (cond != nullptr) cond[r * nc + (j >> 1)] = v;
          if (cond16 != nullptr) cond16[r * ldc16 + (j >> 1)] = f32_to_bf16_rn(v);
        }
      }
    }
    row_tail(r);
  }
}

__global__ void k_base_logprob(const float* __restrict__ y, const float* __restrict__ ld, int64_t n, int d,
                               const float* __restrict__ aux, float* __restrict__ logp) {
  const int lane = threadIdx.x & 31;
  const float c = aux[2 * d];
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < n; r += warps) {
    float s = 0.f;
    for (int j = lane; j < d; j += 32) {
      const float v = y[r * d + j];
      s += v * v;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) {
      // multivariate_normal.logpdf(y, 0, c I) (common.py:285-286)
      logp[r] = ld[r] + (-0.5f * s / c - 0.5f * (float)d * logf(6.283185307179586f * c));
    }
  }
}

__global__ void k_base_sample(const float* __restrict__ z, Rng rng0, int64_t n, int d, const float* __restrict__ aux,
                              float* __restrict__ out) {
  const Rng rng = rng0.at_epoch();
  // jax.random.multivariate_normal(0, c I): mean + z @ cholesky(c I).T = sqrt(c) z
  const float sc = sqrtf(aux[2 * d]);
  const int64_t tot = n * d;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < tot; i += (int64_t)gridDim.x * blockDim.x) {
    float v;
    if (z) {
      v = z[i];
    } else {
      const int64_t r = i / d;
      const int j = (int)(i - r * d);
      const u32x4 b = rng.draw((uint64_t)r, 0, (uint32_t)(j >> 1), RNG_TAG_NF_NORMAL);
      float z0, z1;
      box_muller(b.x, b.y, z0, z1);
      v = (j & 1) ? z1 : z0;
    }
    out[i] = v * sc;
  }
}

static int ew_grid(int64_t tot) {
  int64_t b = (tot + 255) / 256;
  const int64_t cap = (int64_t)sm_count() * 32;
  if (b > cap) b = cap;
  return (int)(b < 1 ? 1 : b);
}

static int rows_grid(int64_t m) {
  int64_t b = (m + 7) / 8;
  const int64_t cap = (int64_t)sm_count() * 16;
  if (b > cap) b = cap;
  return (int)(b < 1 ? 1 : b);
}

// ------------------------------------------------------------------ workspace
struct InferWs {
  int64_t rows;   // chunk rows
  float *xa, *cond, *h0, *h1, *raw, *ld, *ldp;
  int ldp_steps;  // fused spline launches whose log-det partials ldp can hold at once
  uint16_t *cond16, *h16a, *h16b;  // BF16 operands
};

static int64_t align_up(int64_t v, int64_t a) { return (v + a - 1) / a * a; }

// BF16 chunks: 77,824 = 4 x 128 x 152 rows, so that a chunk's 128-row tiles
// fill whole waves of the 152 SMs in the hidden-layer GEMMs (two 256-column
// tiles per row block) and the fused spline kernels (one tile per row block
// and group); measured 2 % faster than 65,536 rows on the 128-D flow's
// global step, 4 % faster than 38,912 rows
constexpr int64_t kBf16ChunkRows = 77824;

// BF16 passes keep the log-det partials of every layer and add them in one
// launch at the end of the pass, for flows of at most kLdMaxSteps layers whose
// partials fit in 512 floats per row (the 128-D, 12-layer, 12-bin flow: 396);
// wider or deeper flows reduce after each layer
static int ldp_steps(const FlowGeom& g, bool bf16) {
  const int64_t per_layer = kSplineEpiPerQuarter * (int64_t)((g.nt_max() + g.spl_dg - 1) / g.spl_dg);
  return (bf16 && g.L <= kLdMaxSteps && per_layer * g.L <= 512) ? g.L : 1;
}

static int64_t infer_floats_per_row(const FlowGeom& g, bool bf16) {
  const int64_t ldp = kSplineEpiPerQuarter * (int64_t)((g.nt_max() + g.spl_dg - 1) / g.spl_dg) * ldp_steps(g, bf16);
  // xa, cond, ld (+ the fused kernel's log-det partials, or the fp32 conditioner buffers)
  return (int64_t)g.d + g.nc_max() + 1 + (bf16 ? ldp : 2 * g.h_max() + (int64_t)g.nt_max() * g.P);
}

static int64_t infer_chunk_rows(const FlowGeom& g, int64_t n, bool bf16) {
  int64_t rows;
  if (bf16) {
    rows = kBf16ChunkRows;
  } else {
    rows = (int64_t)(512ll << 20) / (4 * infer_floats_per_row(g, false));   // ~512 MB of chunk buffers
    rows = rows / 128 * 128;
    if (rows < 128) rows = 128;
    if (rows > 262144) rows = 262144;
  }
  if (n < rows) rows = align_up(n > 0 ? n : 1, 128);
  return rows;
}

static size_t infer_ws_bytes(const FlowGeom& g, int64_t rows, bool bf16) {
  const int64_t f = rows * infer_floats_per_row(g, bf16);
  const int64_t b16 = bf16 ? rows * (align_up(g.nc_max(), 64) + 2 * align_up(g.h_max(), 64)) : 0;
  return (size_t)(4 * f + 2 * b16 + 16 * 256);
}

static void carve_infer(const FlowGeom& g, int64_t rows, bool bf16, void* ws, InferWs& w) {
  char* p = (char*)ws;
  auto take = [&](int64_t bytes) {
    char* r = p;
    p += align_up(bytes, 256);
    return r;
  };
  w.rows = rows;
  w.xa = (float*)take(4 * rows * g.d);
  w.cond = (float*)take(4 * rows * g.nc_max());
  w.ld = (float*)take(4 * rows);
  w.h0 = w.h1 = w.raw = w.ldp = nullptr;
  w.ldp_steps = 0;
  w.cond16 = w.h16a = w.h16b = nullptr;
  if (bf16) {
    w.ldp = (float*)take(4 * rows * kSplineEpiPerQuarter * (int64_t)((g.nt_max() + g.spl_dg - 1) / g.spl_dg) *
                         ldp_steps(g, true));
    w.ldp_steps = ldp_steps(g, true);
    w.cond16 = (uint16_t*)take(2 * rows * align_up(g.nc_max(), 64));
    w.h16a = (uint16_t*)take(2 * rows * align_up(g.h_max(), 64));
    w.h16b = (uint16_t*)take(2 * rows * align_up(g.h_max(), 64));
  } else {
    w.h0 = (float*)take(4 * rows * g.h_max());
    w.h1 = (float*)take(4 * rows * g.h_max());
    w.raw = (float*)take(4 * rows * (int64_t)g.nt_max() * g.P);
  }
}

// conditioner MLP of layer l on rows [0, m): cond (w.cond) -> raw (w.raw)
static int conditioner(const FmcFlow* f, const FlowGeom& g, int l, int64_t m, InferWs& w, cudaStream_t st) {
  const float* th = f->theta + g.layer_off[l];
  const float* a = w.cond;
  int in = g.nc(l);
  float* bufs[2] = {w.h0, w.h1};
  for (int i = 0; i <= g.nh; ++i) {
    const int out = g.lin_out(l, i);
    const float* W = th + g.lin_w(l, i);
    const float* b = th + g.lin_b(l, i);
    float* c = (i == g.nh) ? w.raw : bufs[i & 1];
    int rc = (i == g.nh) ? sgemm<true, true, EPI_BIAS>(st, m, out, in, a, in, W, in, b, nullptr, 0, c, out, 0.f)
                         : sgemm<true, true, EPI_BIAS_TANH>(st, m, out, in, a, in, W, in, b, nullptr, 0, c, out, 0.f);
    if (rc) return rc;
    a = c;
    in = out;
  }
  return FMC_OK;
}

// one pass over all layers for rows x[0, m) -> y, ld (forward or inverse)
static int flow_pass(const FmcFlow* f, const FlowGeom& g, const float* x, float* y, float* ld, int64_t m, bool inverse,
                     InferWs& w, cudaStream_t st) {
  const int grid = rows_grid(m);
  const bool bf16 = f->precision == FMC_PREC_BF16;
  bool folded = false;   // the previous layer's spline kernel applied this layer's affine
  // BF16: the fused spline launches' log-det partials wait in w.ldp (packed,
  // step after step) and are added in one launch -- before the next affine
  // launch that adds to ld, or at the end of the pass -- in the order the
  // per-layer reductions would have added them
  const bool defer = bf16 && w.ldp_steps == g.L;
  LdSteps pend{};
  auto flush = [&]() -> int {
    const int rc = ld_reduce_steps(st, w.ldp, pend, m, ld, g.d, inverse);
    pend.n = 0;
    return rc;
  };
  for (int u = 0; u < g.L; ++u) {
    const int l = inverse ? g.L - 1 - u : u;
    const float* src = (u == 0) ? x : y;
    if (!folded) {
      if (defer && pend.n > 0) {
        const int rc = flush();
        if (rc) return rc;
      }
      // BF16: the conditioning block goes straight to the bf16 GEMM operand
      k_affine<<<grid, 256, 0, st>>>(src, y, bf16 ? nullptr : w.cond, bf16 ? w.cond16 : nullptr, g.w16_cols(l, 0),
                                     m, g.d, g.nc(l), g.cpar(l), f->theta + g.layer_off[l], inverse ? 1 : 0, ld,
                                     u == 0 ? 1 : 0);
      FMC_LAUNCH_CHECK();
    }
    folded = false;
    int rc;
    if (bf16) {
      // hidden layers on tcgen05, then the last Linear fused with the spline,
      // which also applies the next layer's affine where n_dim is even (same
      // bits as that layer's own k_affine launch)
      const uint16_t* h_last = nullptr;
      if ((rc = conditioner_bf16_hidden(f, g, l, m, nullptr, w.cond16, w.h16a, w.h16b, &h_last, st))) return rc;
      const int64_t rows = (m + 127) / 128 * 128;
      SplineFold fold{};
      const SplineFold* fp = nullptr;
      if (u + 1 < g.L && 2 * g.nt(l) == g.d) {
        const int ln = inverse ? l - 1 : l + 1;
        fold.th_next = f->theta + g.layer_off[ln];
        fold.cond16 = w.cond16;
        fold.ldc16 = g.w16_cols(ln, 0);
        fp = &fold;
      }
      if (defer) {
        const int64_t off = pend.n > 0 ? pend.off[pend.n - 1] + (int64_t)pend.parts[pend.n - 1] * m : 0;
        int parts = 0;
        if ((rc = tc_linear_spline(st, g, f, l, h_last, m, rows, inverse, y, nullptr, w.ldp + off, fp, &folded,
                                   &parts)))
          return rc;
        pend.parts[pend.n] = parts;
        pend.off[pend.n] = off;
        pend.th_next[pend.n] = folded ? fold.th_next : nullptr;
        ++pend.n;
      } else if ((rc = tc_linear_spline(st, g, f, l, h_last, m, rows, inverse, y, ld, w.ldp, fp, &folded))) {
        return rc;
      }
    } else {
      if ((rc = conditioner(f, g, l, m, w, st))) return rc;
      if ((rc = launch_spline(g.K, inverse, st, w.raw, y, ld, m, g.d, g.nt(l), g.tpar(l), g.cfg))) return rc;
    }
  }
  return defer ? flush() : FMC_OK;
}

static int check_ws(const FlowGeom& g, int64_t n, bool bf16, void* ws, size_t ws_bytes, int64_t& rows) {
  rows = infer_chunk_rows(g, n, bf16);
  const size_t need = infer_ws_bytes(g, rows, bf16);
  FMC_CHECK_ARG(ws != nullptr && ws_bytes >= need, "workspace of %zu bytes < %zu needed", ws_bytes, need);
  FMC_CHECK_ARG(((uintptr_t)ws & 255) == 0, "workspace must be 256-byte aligned");
  return FMC_OK;
}

static int check_flow_ptrs(const FmcFlow* f) {
  FMC_CHECK_ARG(f->theta != nullptr && f->aux != nullptr, "flow theta/aux is NULL");
  FMC_CHECK_ARG(f->precision == FMC_PREC_FP32 || f->precision == FMC_PREC_BF16, "unknown precision %d", f->precision);
  if (f->precision == FMC_PREC_BF16) FMC_CHECK_ARG(f->theta_bf16 != nullptr, "BF16 mode needs theta_bf16");
  return FMC_OK;
}

// forward/inverse/log_prob driver over row chunks
enum PassKind { PASS_FORWARD, PASS_INVERSE, PASS_LOGPROB };

int flow_apply(const FmcFlow* f, const float* x, int64_t n, float* out, float* out_ld, PassKind kind, void* ws,
               size_t ws_bytes, cudaStream_t st) {
  FlowGeom g;
  int rc = make_geom(f, g);
  if (rc) return rc;
  if ((rc = check_flow_ptrs(f))) return rc;
  FMC_CHECK_ARG(n >= 0, "n < 0");
  if (n == 0) return FMC_OK;
  FMC_CHECK_ARG(x != nullptr && out != nullptr, "NULL array");
  int64_t rows;
  const bool bf16 = f->precision == FMC_PREC_BF16;
  if ((rc = check_ws(g, n, bf16, ws, ws_bytes, rows))) return rc;
  InferWs w;
  carve_infer(g, rows, bf16, ws, w);
  for (int64_t r0 = 0; r0 < n; r0 += rows) {
    const int64_t m = (n - r0 < rows) ? n - r0 : rows;
    const float* xc = x + r0 * g.d;
    if (kind == PASS_LOGPROB) {
      k_standardize<<<ew_grid(m * g.d), 256, 0, st>>>(xc, m, g.d, f->aux, w.xa);
      FMC_LAUNCH_CHECK();
      if ((rc = flow_pass(f, g, w.xa, w.xa, w.ld, m, false, w, st))) return rc;
      k_base_logprob<<<rows_grid(m), 256, 0, st>>>(w.xa, w.ld, m, g.d, f->aux, out + r0);
      FMC_LAUNCH_CHECK();
    } else {
      float* yc = out + r0 * g.d;
      float* ldc = out_ld ? out_ld + r0 : w.ld;
      if ((rc = flow_pass(f, g, xc, yc, ldc, m, kind == PASS_INVERSE, w, st))) return rc;
    }
  }
  return FMC_OK;
}

int flow_sample(const FmcFlow* f, uint64_t seed, uint64_t counter, const float* z, int64_t n, float* x, void* ws,
                size_t ws_bytes, cudaStream_t st) {
  FlowGeom g;
  int rc = make_geom(f, g);
  if (rc) return rc;
  if ((rc = check_flow_ptrs(f))) return rc;
  FMC_CHECK_ARG(n >= 0, "n < 0");
  if (n == 0) return FMC_OK;
  FMC_CHECK_ARG(x != nullptr, "NULL output");
  int64_t rows;
  const bool bf16 = f->precision == FMC_PREC_BF16;
  if ((rc = check_ws(g, n, bf16, ws, ws_bytes, rows))) return rc;
  InferWs w;
  carve_infer(g, rows, bf16, ws, w);
  const Rng rng{(uint32_t)seed, (uint32_t)(seed >> 32), counter, rng_epoch()};
  k_base_sample<<<ew_grid(n * g.d), 256, 0, st>>>(z, rng, n, g.d, f->aux, x);
  FMC_LAUNCH_CHECK();
  for (int64_t r0 = 0; r0 < n; r0 += rows) {
    const int64_t m = (n - r0 < rows) ? n - r0 : rows;
    float* xc = x + r0 * g.d;
    if ((rc = flow_pass(f, g, xc, xc, w.ld, m, true, w, st))) return rc;
  }
  k_destandardize<<<ew_grid(n * g.d), 256, 0, st>>>(x, n, g.d, f->aux);
  FMC_LAUNCH_CHECK();
  return FMC_OK;
}

int flow_apply_logprob(const FmcFlow* f, const float* x, int64_t n, float* logp, void* ws, size_t ws_bytes,
                       cudaStream_t st) {
  return flow_apply(f, x, n, logp, nullptr, PASS_LOGPROB, ws, ws_bytes, st);
}

int flow_sample_rows(const FmcFlow* f, uint64_t seed, uint64_t counter, const float* z, int64_t n, float* x, void* ws,
                     size_t ws_bytes, cudaStream_t st) {
  return flow_sample(f, seed, counter, z, n, x, ws, ws_bytes, st);
}

size_t flow_infer_ws_bytes(const FmcFlow* f, int64_t n) {
  FlowGeom g;
  if (make_geom(f, g) != FMC_OK) return 0;
  const bool bf16 = f->precision == FMC_PREC_BF16;
  return infer_ws_bytes(g, infer_chunk_rows(g, n, bf16), bf16);
}


}  // namespace fmc

using namespace fmc;

extern "C" int fmc_flow_layout(const FmcFlow* flow, int64_t* n_params, int64_t* layer_offsets) {
  FlowGeom g;
  int rc = make_geom(flow, g);
  if (rc) return rc;
  if (n_params) *n_params = g.n_params;
  if (layer_offsets)
    for (int l = 0; l <= g.L; ++l) layer_offsets[l] = g.layer_off[l];
  return FMC_OK;
}

extern "C" int fmc_flow_workspace_size(const FmcFlow* flow, int64_t n, int32_t mode, size_t* bytes) {
  FlowGeom g;
  int rc = make_geom(flow, g);
  if (rc) return rc;
  FMC_CHECK_ARG(bytes != nullptr, "bytes is NULL");
  FMC_CHECK_ARG(n >= 0, "n < 0");
  if (mode == 0) {
    const bool bf16 = flow->precision == FMC_PREC_BF16;
    *bytes = infer_ws_bytes(g, infer_chunk_rows(g, n, bf16), bf16);
  } else if (mode == 1) {
    *bytes = train_ws_bytes(g, n, flow->precision == FMC_PREC_BF16);
  } else {
    set_error("unknown workspace mode %d", mode);
    return FMC_ERR_INVALID_ARG;
  }
  return FMC_OK;
}

extern "C" int fmc_flow_sync_bf16(const FmcFlow* flow, void* stream) {
  FlowGeom g;
  int rc = make_geom(flow, g);
  if (rc) return rc;
  FMC_CHECK_ARG(flow->theta && flow->theta_bf16, "theta/theta_bf16 NULL");
  return pack_bf16_weights(g, flow->theta, flow->theta_bf16, (cudaStream_t)stream);
}

extern "C" int fmc_flow_bf16_size(const FmcFlow* flow, int64_t* n_elems) {
  FlowGeom g;
  int rc = make_geom(flow, g);
  if (rc) return rc;
  FMC_CHECK_ARG(n_elems != nullptr, "n_elems is NULL");
  *n_elems = g.n_w16;
  return FMC_OK;
}

extern "C" int fmc_flow_forward(const FmcFlow* flow, const float* x, int64_t n, float* y, float* logdet, void* ws,
                                size_t ws_bytes, void* stream) {
  return flow_apply(flow, x, n, y, logdet, PASS_FORWARD, ws, ws_bytes, (cudaStream_t)stream);
}

extern "C" int fmc_flow_inverse(const FmcFlow* flow, const float* z, int64_t n, float* x, float* logdet, void* ws,
                                size_t ws_bytes, void* stream) {
  return flow_apply(flow, z, n, x, logdet, PASS_INVERSE, ws, ws_bytes, (cudaStream_t)stream);
}

extern "C" int fmc_flow_log_prob(const FmcFlow* flow, const float* x, int64_t n, float* logp, void* ws,
                                 size_t ws_bytes, void* stream) {
  return flow_apply(flow, x, n, logp, nullptr, PASS_LOGPROB, ws, ws_bytes, (cudaStream_t)stream);
}

extern "C" int fmc_flow_sample(const FmcFlow* flow, uint64_t seed, uint64_t counter, const float* z, int64_t n,
                               float* x, void* ws, size_t ws_bytes, void* stream) {
  return flow_sample(flow, seed, counter, z, n, x, ws, ws_bytes, (cudaStream_t)stream);
}
