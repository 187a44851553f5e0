// realnvp.cu -- the RealNVP flow (resource/model/nf_model/realNVP.py of flowMC).
//
// A layer is MaskedCouplingLayer(MLPAffine(scale_MLP, shift_MLP, dt), m)
// (realNVP.py:163-176, common.py:127-208):
//   c = x * m,   s = tanh(MLP_s(c)) * dt,   t = MLP_t(c) * dt
//   y = (1 - m) * ((x + t) * exp(s)) + m * x,   log-det = sum (1 - m) * s
// with MLP = Linear(d, H), relu, Linear(H, d). The masks are float leaves of
// the reference model, so optax's weight decay moves them off 0/1; they live
// in aux and every kernel uses the general formula.
//
// Per layer and row block: the first Linears of both MLPs as one GEMM
// (W1 = [W1s; W1t], relu epilogue), the two second Linears as GEMMs with
// bias epilogues, then one warp per row applies the coupling and sums the
// log-det. The backward recomputes a layer's activations from its stored
// input, runs the coupling adjoint elementwise, the two relu-masked dH GEMMs
// and the dc GEMM, and forms the weight and bias gradients as split-K
// GEMMs over the batch (fixed-order slice sums: deterministic). FP32 SIMT
// GEMMs throughout: RealNVP's MLPs are narrow [d, H, d].
#include "flow.cuh"
#include "gemm_simt.cuh"

namespace fmc {

struct RnvpGeom {
  int d, L, H;
  float dt;
  int64_t off_b1, off_W2s, off_b2s, off_W2t, off_b2t, per_layer, n_params, n_aux;
};

static int rnvp_geom(const FmcRealNVP* f, RnvpGeom& g) {
  FMC_CHECK_ARG(f != nullptr, "flow is NULL");
  FMC_CHECK_ARG(f->n_dim >= 1 && f->n_layers >= 1 && f->n_hidden >= 1, "RealNVP shape d=%d L=%d H=%d", f->n_dim,
                f->n_layers, f->n_hidden);
  g.d = f->n_dim;
  g.L = f->n_layers;
  g.H = f->n_hidden;
  g.dt = f->dt;
  const int64_t d = g.d, H = g.H;
  g.off_b1 = 2 * H * d;
  g.off_W2s = g.off_b1 + 2 * H;
  g.off_b2s = g.off_W2s + d * H;
  g.off_W2t = g.off_b2s + d;
  g.off_b2t = g.off_W2t + d * H;
  g.per_layer = g.off_b2t + d;
  g.n_params = g.per_layer * g.L;
  g.n_aux = 2 * d + 2 + (int64_t)g.L * d;
  return FMC_OK;
}

constexpr int64_t kRnvpChunk = 65536;   // rows per inference chunk
constexpr int kMaxSlices = kKouterMaxSlices;   // split-K slices of the weight gradients

static int grid_for(int64_t tot, int per_sm = 8) {
  int64_t b = (tot + 255) / 256;
  const int64_t cap = (int64_t)sm_count() * per_sm;
  if (b > cap) b = cap;
  return (int)(b < 1 ? 1 : b);
}

static int warp_grid(int64_t rows) {
  int64_t b = (rows + 7) / 8;   // 8 warps per 256-thread block
  const int64_t cap = (int64_t)sm_count() * 16;
  if (b > cap) b = cap;
  return (int)(b < 1 ? 1 : b);
}

// ------------------------------------------------------------------ kernels
__global__ void k_rnvp_cond(const float* __restrict__ x, const float* __restrict__ m, int64_t n, int d,
                            float* __restrict__ cond) {
  const int64_t tot = n * d;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < tot; i += (int64_t)gridDim.x * blockDim.x)
    cond[i] = x[i] * m[i % d];
}

// one warp per row; y may alias x. first: ld = sum, else ld += sum
__global__ void k_rnvp_couple(const float* x, const float* __restrict__ sraw, const float* __restrict__ tt,
                              const float* __restrict__ m, int64_t n, int d, float dt, int inverse, float* y,
                              float* __restrict__ ld, int first) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < n; r += warps) {
    float acc = 0.f;
    for (int j = lane; j < d; j += 32) {
      const int64_t e = r * d + j;
      const float mj = m[j], xv = x[e];
      const float s = tanhf(sraw[e]) * dt;        // MLPAffine: tanh(scale_MLP(c)) * dt
      const float t = tt[e] * dt;                 //            shift_MLP(c) * dt
      const float ya = inverse ? xv * expf(-s) - t : (xv + t) * expf(s);
      y[e] = (1.f - mj) * ya + mj * xv;           // MaskedCouplingLayer mix
      acc += (1.f - mj) * s;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) {
      const float v = inverse ? -acc : acc;
      ld[r] = first ? v : ld[r] + v;
    }
  }
}

// adjoint of one forward coupling: gy (dL/dy) and gld (dL/d log-det, the
// same for every row) -> gx (the direct part; the conditioner's part is
// added later), and in place sraw -> dL/d sraw, tt -> dL/d tt
__global__ void k_rnvp_couple_bwd(const float* __restrict__ x, float* __restrict__ sraw, float* __restrict__ tt,
                                  const float* __restrict__ m, const float* __restrict__ gy, int64_t n, int d,
                                  float dt, float gld, float* __restrict__ gx) {
  const int64_t tot = n * d;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
    const float mj = m[e % d], xv = x[e];
    const float th = tanhf(sraw[e]);
    const float s = th * dt, t = tt[e] * dt;
    const float ex = expf(s);
    const float ya = (xv + t) * ex;
    const float g = gy[e];
    const float dya = (1.f - mj) * g;
    gx[e] = mj * g + dya * ex;
    const float ds = dya * ya + gld * (1.f - mj);
    sraw[e] = ds * dt * (1.f - th * th);
    tt[e] = dya * ex * dt;
  }
}

__global__ void k_rnvp_add_masked(float* __restrict__ gx, const float* __restrict__ dc, const float* __restrict__ m,
                                  int64_t n, int d) {
  const int64_t tot = n * d;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x)
    gx[e] += dc[e] * m[e % d];
}

// log N(y; 0, I) + ld (realNVP.py:218-221: the standard normal, not the base distribution)
__global__ void k_rnvp_logprob(const float* __restrict__ y, const float* __restrict__ ld, int64_t n, int d,
                               float* __restrict__ logp) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < n; r += warps) {
    float s = 0.f;
    for (int j = lane; j < d; j += 32) {
      const float v = y[r * d + j];
      s += v * v;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) logp[r] = ld[r] + (-0.5f * s - 0.5f * (float)d * logf(6.283185307179586f));
  }
}

// loss = -mean(logp) in fixed order (one block); gy = y / n seeds the backward
__global__ void k_rnvp_loss(const float* __restrict__ logp, int64_t n, float* __restrict__ loss) {
  __shared__ float sh[32];
  float s = 0.f;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s += logp[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    float v = (threadIdx.x < (blockDim.x >> 5)) ? sh[threadIdx.x] : 0.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) *loss = -v / (float)n;
  }
}

__global__ void k_rnvp_scale(const float* __restrict__ y, int64_t tot, float c, float* __restrict__ out) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x)
    out[e] = y[e] * c;
}

// ------------------------------------------------------------------ layer passes
struct RnvpScratch {
  float* cond;   // [rows, d]
  float* h;      // [rows, 2H]
  float* sraw;   // [rows, d]
  float* tt;     // [rows, d]
};

static const float* layer_mask(const RnvpGeom& g, const float* aux, int l) { return aux + 2 * g.d + 2 + (int64_t)l * g.d; }

// the layer's conditioner: cond = x * m, h = relu(cond W1^T + b1), sraw, tt
static int rnvp_conditioner(cudaStream_t st, const RnvpGeom& g, const float* th, const float* m, const float* x,
                            int64_t rows, const RnvpScratch& s) {
  const int d = g.d, H = g.H;
  k_rnvp_cond<<<grid_for(rows * d), 256, 0, st>>>(x, m, rows, d, s.cond);
  FMC_LAUNCH_CHECK();
  int rc = sgemm<true, true, EPI_BIAS_RELU>(st, rows, 2 * H, d, s.cond, d, th, d, th + g.off_b1, nullptr, 0, s.h,
                                            2 * H, 0.f);
  if (rc) return rc;
  rc = sgemm<true, true, EPI_BIAS>(st, rows, d, H, s.h, 2 * H, th + g.off_W2s, H, th + g.off_b2s, nullptr, 0, s.sraw,
                                   d, 0.f);
  if (rc) return rc;
  return sgemm<true, true, EPI_BIAS>(st, rows, d, H, s.h + H, 2 * H, th + g.off_W2t, H, th + g.off_b2t, nullptr, 0,
                                     s.tt, d, 0.f);
}

// all layers, in place on x [rows, d] (forward: 0..L-1, inverse: L-1..0); ld = the summed log-det
static int rnvp_pass(cudaStream_t st, const RnvpGeom& g, const FmcRealNVP* f, float* x, int64_t rows, float* ld,
                     bool inverse, const RnvpScratch& s) {
  for (int i = 0; i < g.L; ++i) {
    const int l = inverse ? g.L - 1 - i : i;
    const float* th = f->theta + (int64_t)l * g.per_layer;
    const float* m = layer_mask(g, f->aux, l);
    int rc = rnvp_conditioner(st, g, th, m, x, rows, s);
    if (rc) return rc;
    k_rnvp_couple<<<warp_grid(rows), 256, 0, st>>>(x, s.sraw, s.tt, m, rows, g.d, g.dt, inverse ? 1 : 0, x, ld,
                                                   i == 0 ? 1 : 0);
    FMC_LAUNCH_CHECK();
  }
  return FMC_OK;
}

static size_t infer_floats(const RnvpGeom& g, int64_t rows) {
  return (size_t)rows * (4 * (size_t)g.d + 2 * (size_t)g.H) + (size_t)rows + 64;
}

static int carve_infer(const RnvpGeom& g, int64_t rows, void* ws, size_t ws_bytes, RnvpScratch& s, float** xa,
                       float** ld) {
  FMC_CHECK_ARG(ws != nullptr && ws_bytes >= infer_floats(g, rows) * sizeof(float),
                "workspace of %zu bytes is smaller than fmc_rnvp_workspace_size", ws_bytes);
  float* p = (float*)ws;
  s.cond = p; p += rows * g.d;
  s.h = p; p += rows * 2 * (int64_t)g.H;
  s.sraw = p; p += rows * g.d;
  s.tt = p; p += rows * g.d;
  *xa = p; p += rows * g.d;
  *ld = p;
  return FMC_OK;
}

static int64_t train_part_floats(const RnvpGeom& g) {
  return (int64_t)kMaxSlices * 2 * g.H * (int64_t)g.d;
}

static size_t train_floats(const RnvpGeom& g, int64_t n) {
  const size_t d = g.d, H = g.H;
  return (size_t)n * ((g.L + 1) * d + 6 * d + 4 * H + 2) + (size_t)train_part_floats(g) + 64;
}

}  // namespace fmc

using namespace fmc;

extern "C" int fmc_rnvp_layout(const FmcRealNVP* flow, int64_t* n_params, int64_t* n_aux) {
  RnvpGeom g;
  int rc = rnvp_geom(flow, g);
  if (rc) return rc;
  if (n_params) *n_params = g.n_params;
  if (n_aux) *n_aux = g.n_aux;
  return FMC_OK;
}

extern "C" int fmc_rnvp_workspace_size(const FmcRealNVP* flow, int64_t n, int32_t mode, size_t* bytes) {
  RnvpGeom g;
  int rc = rnvp_geom(flow, g);
  if (rc) return rc;
  FMC_CHECK_ARG(bytes != nullptr && n >= 0, "bad arguments");
  const int64_t rows = n < kRnvpChunk ? (n > 0 ? n : 1) : kRnvpChunk;
  *bytes = (mode == 1 ? train_floats(g, n > 0 ? n : 1) : infer_floats(g, rows)) * sizeof(float);
  return FMC_OK;
}

static int rnvp_transform(const FmcRealNVP* flow, const float* in, int64_t n, float* out, float* logdet, void* ws,
                          size_t ws_bytes, void* stream, bool inverse) {
  RnvpGeom g;
  int rc = rnvp_geom(flow, g);
  if (rc) return rc;
  FMC_CHECK_ARG(n >= 0, "n < 0");
  if (n == 0) return FMC_OK;
  FMC_CHECK_ARG(in && out && logdet && flow->theta && flow->aux, "NULL array argument");
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t rows = n < kRnvpChunk ? n : kRnvpChunk;
  RnvpScratch s;
  float *xa, *ldw;
  rc = carve_infer(g, rows, ws, ws_bytes, s, &xa, &ldw);
  if (rc) return rc;
  if (out != in) FMC_CUDA_TRY(cudaMemcpyAsync(out, in, sizeof(float) * n * g.d, cudaMemcpyDeviceToDevice, st));
  for (int64_t r0 = 0; r0 < n; r0 += rows) {
    const int64_t m = (n - r0 < rows) ? n - r0 : rows;
    rc = rnvp_pass(st, g, flow, out + r0 * g.d, m, logdet + r0, inverse, s);
    if (rc) return rc;
  }
  return FMC_OK;
}

extern "C" int fmc_rnvp_forward(const FmcRealNVP* flow, const float* x, int64_t n, float* y, float* logdet, void* ws,
                                size_t ws_bytes, void* stream) {
  return rnvp_transform(flow, x, n, y, logdet, ws, ws_bytes, stream, false);
}

extern "C" int fmc_rnvp_inverse(const FmcRealNVP* flow, const float* y, int64_t n, float* x, float* logdet, void* ws,
                                size_t ws_bytes, void* stream) {
  return rnvp_transform(flow, y, n, x, logdet, ws, ws_bytes, stream, true);
}

extern "C" int fmc_rnvp_log_prob(const FmcRealNVP* flow, const float* x, int64_t n, float* logp, void* ws,
                                 size_t ws_bytes, void* stream) {
  RnvpGeom g;
  int rc = rnvp_geom(flow, g);
  if (rc) return rc;
  FMC_CHECK_ARG(n >= 0, "n < 0");
  if (n == 0) return FMC_OK;
  FMC_CHECK_ARG(x && logp && flow->theta && flow->aux, "NULL array argument");
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t rows = n < kRnvpChunk ? n : kRnvpChunk;
  RnvpScratch s;
  float *xa, *ld;
  rc = carve_infer(g, rows, ws, ws_bytes, s, &xa, &ld);
  if (rc) return rc;
  for (int64_t r0 = 0; r0 < n; r0 += rows) {
    const int64_t m = (n - r0 < rows) ? n - r0 : rows;
    k_standardize<<<grid_for(m * g.d), 256, 0, st>>>(x + r0 * g.d, m, g.d, flow->aux, xa);
    FMC_LAUNCH_CHECK();
    rc = rnvp_pass(st, g, flow, xa, m, ld, false, s);
    if (rc) return rc;
    k_rnvp_logprob<<<warp_grid(m), 256, 0, st>>>(xa, ld, m, g.d, logp + r0);
    FMC_LAUNCH_CHECK();
  }
  return FMC_OK;
}

extern "C" int fmc_rnvp_sample(const FmcRealNVP* flow, uint64_t seed, uint64_t counter, const float* z, int64_t n,
                               float* out, void* ws, size_t ws_bytes, void* stream) {
  RnvpGeom g;
  int rc = rnvp_geom(flow, g);
  if (rc) return rc;
  FMC_CHECK_ARG(n >= 0, "n < 0");
  if (n == 0) return FMC_OK;
  FMC_CHECK_ARG(out && flow->theta && flow->aux, "NULL array argument");
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t rows = n < kRnvpChunk ? n : kRnvpChunk;
  RnvpScratch s;
  float *xa, *ld;
  rc = carve_infer(g, rows, ws, ws_bytes, s, &xa, &ld);
  if (rc) return rc;
  // base_dist.sample: sqrt(c) z for the Gaussian(0, c I) base (common.py:288-293)
  const Rng rng{(uint32_t)seed, (uint32_t)(seed >> 32), counter, rng_epoch()};
  k_base_sample<<<grid_for(n * g.d), 256, 0, st>>>(z, rng, n, g.d, flow->aux, out);
  FMC_LAUNCH_CHECK();
  for (int64_t r0 = 0; r0 < n; r0 += rows) {
    const int64_t m = (n - r0 < rows) ? n - r0 : rows;
    rc = rnvp_pass(st, g, flow, out + r0 * g.d, m, ld, true, s);
    if (rc) return rc;
  }
  k_destandardize<<<grid_for(n * g.d), 256, 0, st>>>(out, n, g.d, flow->aux);
  FMC_LAUNCH_CHECK();
  return FMC_OK;
}

extern "C" int fmc_rnvp_loss_grad(const FmcRealNVP* flow, const float* x, int64_t n, float* loss, float* grad,
                                  void* ws, size_t ws_bytes, void* stream) {
  RnvpGeom g;
  int rc = rnvp_geom(flow, g);
  if (rc) return rc;
  FMC_CHECK_ARG(n >= 1, "n=%lld < 1", (long long)n);
  FMC_CHECK_ARG(x && loss && grad && flow->theta && flow->aux, "NULL array argument");
  FMC_CHECK_ARG(ws != nullptr && ws_bytes >= train_floats(g, n) * sizeof(float),
                "workspace of %zu bytes is smaller than fmc_rnvp_workspace_size", ws_bytes);
  cudaStream_t st = (cudaStream_t)stream;
  const int d = g.d, H = g.H;
  float* p = (float*)ws;
  float* X = p; p += (int64_t)(g.L + 1) * n * d;   // layer inputs, X[L] = y
  RnvpScratch s;
  s.cond = p; p += n * d;
  s.h = p; p += n * 2 * (int64_t)H;
  s.sraw = p; p += n * d;
  s.tt = p; p += n * d;
  float* gy = p; p += n * d;
  float* gx = p; p += n * d;
  float* dh = p; p += n * 2 * (int64_t)H;
  float* dc = p; p += n * d;
  float* ld = p; p += n;
  float* logp = p; p += n;
  float* part = p;
  const int64_t part_floats = train_part_floats(g);

  // forward, keeping every layer's input
  k_standardize<<<grid_for(n * d), 256, 0, st>>>(x, n, d, flow->aux, X);
  FMC_LAUNCH_CHECK();
  for (int l = 0; l < g.L; ++l) {
    const float* th = flow->theta + (int64_t)l * g.per_layer;
    const float* m = layer_mask(g, flow->aux, l);
    const float* xl = X + (int64_t)l * n * d;
    float* xn = X + (int64_t)(l + 1) * n * d;
    rc = rnvp_conditioner(st, g, th, m, xl, n, s);
    if (rc) return rc;
    k_rnvp_couple<<<warp_grid(n), 256, 0, st>>>(xl, s.sraw, s.tt, m, n, d, g.dt, 0, xn, ld, l == 0 ? 1 : 0);
    FMC_LAUNCH_CHECK();
  }
  float* y = X + (int64_t)g.L * n * d;
  k_rnvp_logprob<<<warp_grid(n), 256, 0, st>>>(y, ld, n, d, logp);
  FMC_LAUNCH_CHECK();
  k_rnvp_loss<<<1, 1024, 0, st>>>(logp, n, loss);
  FMC_LAUNCH_CHECK();

  // backward: loss = -mean(ld + log N(y)) -> dL/dy = y / n, dL/d ld = -1 / n
  k_rnvp_scale<<<grid_for(n * d), 256, 0, st>>>(y, n * d, 1.f / (float)n, gy);
  FMC_LAUNCH_CHECK();
  const float gld = -1.f / (float)n;
  for (int l = g.L - 1; l >= 0; --l) {
    const float* th = flow->theta + (int64_t)l * g.per_layer;
    float* gth = grad + (int64_t)l * g.per_layer;
    const float* m = layer_mask(g, flow->aux, l);
    const float* xl = X + (int64_t)l * n * d;
    rc = rnvp_conditioner(st, g, th, m, xl, n, s);
    if (rc) return rc;
    k_rnvp_couple_bwd<<<grid_for(n * d), 256, 0, st>>>(xl, s.sraw, s.tt, m, gy, n, d, g.dt, gld, gx);
    FMC_LAUNCH_CHECK();
    // dH = [dsraw W2s, dtt W2t] masked by relu'
    rc = sgemm<true, false, EPI_DRELU>(st, n, H, d, s.sraw, d, th + g.off_W2s, H, nullptr, s.h, 2 * H, dh, 2 * H, 0.f);
    if (rc) return rc;
    rc = sgemm<true, false, EPI_DRELU>(st, n, H, d, s.tt, d, th + g.off_W2t, H, nullptr, s.h + H, 2 * H, dh + H,
                                       2 * H, 0.f);
    if (rc) return rc;
    // dc = dH W1; gx += dc * m
    rc = sgemm<true, false, EPI_NONE>(st, n, d, 2 * H, dh, 2 * H, th, d, nullptr, nullptr, 0, dc, d, 0.f);
    if (rc) return rc;
    k_rnvp_add_masked<<<grid_for(n * d), 256, 0, st>>>(gx, dc, m, n, d);
    FMC_LAUNCH_CHECK();
    // weight and bias gradients over the batch
    rc = kouter(st, d, H, n, s.sraw, d, s.h, 2 * H, false, part, part_floats, gth + g.off_W2s);
    if (rc) return rc;
    rc = kouter(st, d, 1, n, s.sraw, d, nullptr, 0, true, part, part_floats, gth + g.off_b2s);
    if (rc) return rc;
    rc = kouter(st, d, H, n, s.tt, d, s.h + H, 2 * H, false, part, part_floats, gth + g.off_W2t);
    if (rc) return rc;
    rc = kouter(st, d, 1, n, s.tt, d, nullptr, 0, true, part, part_floats, gth + g.off_b2t);
    if (rc) return rc;
    rc = kouter(st, 2 * H, d, n, dh, 2 * H, s.cond, d, false, part, part_floats, gth);
    if (rc) return rc;
    rc = kouter(st, 2 * H, 1, n, dh, 2 * H, nullptr, 0, true, part, part_floats, gth + g.off_b1);
    if (rc) return rc;
    float* t = gy;
    gy = gx;
    gx = t;
  }
  return FMC_OK;
}
