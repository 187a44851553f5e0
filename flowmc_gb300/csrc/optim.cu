// optim.cu -- device side of NFModel.train / TrainModel without host syncs.
//
//  * fmc_adamw_step: optax.chain(clip_by_global_norm(max_norm),
//    adamw(lr, b1, b2, eps, weight_decay)) + apply_updates
//    (resource/optimizer.py:19-22, nf_model/base.py:123-124), written from
//    Loshchilov & Hutter (2019) / Kingma & Ba (2015) and optax's documented
//    defaults. Two launches: a fixed-order sum of squares, then the update.
//  * fmc_flag_less / fmc_copy_if: best-epoch model selection
//    (nf_model/base.py:196-200) as device predicates.
//  * fmc_column_stats: data_mean / diag(data_cov) (nf_model/base.py:187-188).
//  * fmc_permute_rows: batch gather under a pseudo-random permutation
//    (jax.random.permutation, nf_model/base.py:141-146): a 4-round Feistel
//    network on the next power of two with cycle walking (Black & Rogaway,
//    "Ciphers with arbitrary finite domains", CT-RSA 2002).
//  * fmc_select_training_data: TrainModel's finite-row filter, per-chain
//    history window and with-replacement resampling (train_model.py:66-80).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <mutex>
#include "common.cuh"
#include "gemm_tc.cuh"

namespace fmc {

template <int NT>
__device__ __forceinline__ float block_sum_f(float v, float* sh) {
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
  return r;
}

constexpr int kNormBlocks = 512;

__global__ void __launch_bounds__(256) k_sumsq(const float* __restrict__ g, int64_t n, float* __restrict__ part) {
  __shared__ float sh[32];
  float s = 0.f;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float v = g[i];
    s += v * v;
  }
  s = block_sum_f<256>(s, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// state[0] = clip factor applied as (g / norm) * max_norm, state[1] = norm; count += 1
__global__ void k_norm_final(const float* __restrict__ part, int nb, float max_norm, float* __restrict__ state,
                             int32_t* __restrict__ count) {
  if (threadIdx.x != 0) return;
  float s = 0.f;
  for (int b = 0; b < nb; ++b) s += part[b];
  const float norm = sqrtf(s);
  state[0] = (norm < max_norm) ? 0.f : 1.f;  // 1 -> clip
  state[1] = norm;
  *count += 1;
}

__global__ void __launch_bounds__(256) k_adamw(float* __restrict__ theta, uint16_t* __restrict__ theta16,
                                               const float* __restrict__ grad, float* __restrict__ m,
                                               float* __restrict__ v, int64_t n, const float* __restrict__ state,
                                               const int32_t* __restrict__ count, float lr, float b1, float b2,
                                               float eps, float wd, float max_norm, float* __restrict__ aux,
                                               int n_aux) {
  const bool clip = state[0] != 0.f;
  const float norm = state[1];
  const float t = (float)*count;
  const float bc1 = 1.f - powf(b1, t), bc2 = 1.f - powf(b2, t);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float g = grad[i];
    if (clip) g = (g / norm) * max_norm;
    const float mi = (1.f - b1) * g + b1 * m[i];
    const float vi = (1.f - b2) * (g * g) + b2 * v[i];
    m[i] = mi;
    v[i] = vi;
    const float u = (mi / bc1) / (sqrtf(vi / bc2) + eps) + wd * theta[i];
    const float th = theta[i] + (-lr * u);
    theta[i] = th;
    if (theta16) theta16[i] = f32_to_bf16_rn(th);
  }
  // float leaves with zero gradient (data_mean, data_cov, base covariance, ...):
  // m = v = 0 so the update is the weight decay alone
  if (aux && blockIdx.x == 0) {
    for (int i = threadIdx.x; i < n_aux; i += blockDim.x) aux[i] = aux[i] + (-lr * (wd * aux[i]));
  }
}

__global__ void k_flag_less(const float* __restrict__ a, float* __restrict__ best, int32_t* __restrict__ flag) {
  if (threadIdx.x == 0) {
    const bool lt = *a < *best;   // nf_model/base.py:197 (NaN compares false)
    *flag = lt ? 1 : 0;
    if (lt) *best = *a;
  }
}

__global__ void k_copy_if(const int32_t* __restrict__ flag, const uint4* __restrict__ src, uint4* __restrict__ dst,
                          int64_t n16, const uint8_t* __restrict__ src_tail, uint8_t* __restrict__ dst_tail,
                          int tail) {
  if (*flag == 0) return;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n16; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
  if (blockIdx.x == 0 && threadIdx.x < tail) dst_tail[threadIdx.x] = src_tail[threadIdx.x];
}

// Column mean and unbiased variance of x [n, d] in two deterministic stages:
// row block b (rows [b*rows_per, ...)) computes, per column, its own mean and
// sum of squared deviations (two passes over its rows, coalesced across the
// column); the final kernel merges the blocks in index order with the
// pairwise update of Chan, Golub and LeVeque (1979):
//   n = na + nb, delta = mb - ma, m = ma + delta nb / n, M2 = M2a + M2b + delta^2 na nb / n.
// Partials live in the caller's workspace (one column tile at a time):
// 2 * kColStatBlocks * min(d, kColStatCols) floats.
constexpr int kColStatBlocks = 512;
constexpr int kColStatCols = 512;

// x points at the tile's first column; row stride d, tile width dc
__global__ void k_colstat_partial(const float* __restrict__ x, int64_t n, int d, int dc, int64_t rows_per,
                                  float* __restrict__ pmean, float* __restrict__ pm2) {
  const int j = blockIdx.y * blockDim.x + threadIdx.x;
  if (j >= dc) return;
  const int64_t r0 = blockIdx.x * rows_per;
  const int64_t r1 = (r0 + rows_per < n) ? r0 + rows_per : n;
  float s = 0.f;
  for (int64_t r = r0; r < r1; ++r) s += x[r * d + j];
  const float mu = r1 > r0 ? s / (float)(r1 - r0) : 0.f;
  float q = 0.f;
  for (int64_t r = r0; r < r1; ++r) {
    const float e = x[r * d + j] - mu;
    q += e * e;
  }
  pmean[(int64_t)blockIdx.x * dc + j] = mu;
  pm2[(int64_t)blockIdx.x * dc + j] = q;
}

__global__ void k_colstat_final(const float* __restrict__ pmean, const float* __restrict__ pm2, int rb, int64_t n,
                                int d, int64_t rows_per, float* __restrict__ mean, float* __restrict__ var) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= d) return;
  double na = 0.0, ma = 0.0, m2 = 0.0;
  for (int b = 0; b < rb; ++b) {
    const int64_t r0 = b * rows_per;
    const int64_t r1 = (r0 + rows_per < n) ? r0 + rows_per : n;
    const double nb = (double)(r1 - r0);
    if (nb <= 0.0) continue;
    const double mb = pmean[(int64_t)b * d + j], qb = pm2[(int64_t)b * d + j];
    const double nn = na + nb, delta = mb - ma;
    ma += delta * nb / nn;
    m2 += qb + delta * delta * na * nb / nn;
    na = nn;
  }
  mean[j] = (float)ma;
  var[j] = (float)(m2 / (double)(n - 1));
}

// ---------------------------------------------------------------- Feistel permutation
struct Perm {
  uint64_t n;
  int half_bits;  // bits per Feistel half (domain = 4^half_bits >= n)
  uint32_t k[4];
  const uint64_t* epoch;  // folded into the round keys (rng_epoch)
  __device__ __forceinline__ Perm at_epoch() const {
    Perm p = *this;
    if (epoch != nullptr) {
      const uint64_t e = mix64(*epoch), f = e ? mix64(e ^ 0x9E3779B97F4A7C15ull) : 0ull;
      p.k[0] ^= (uint32_t)e;
      p.k[1] ^= (uint32_t)(e >> 32);
      p.k[2] ^= (uint32_t)f;
      p.k[3] ^= (uint32_t)(f >> 32);
    }
    return p;
  }
  __device__ __forceinline__ uint64_t round_once(uint64_t v) const {
    const uint32_t mask = (half_bits >= 32) ? 0xffffffffu : ((1u << half_bits) - 1u);
    uint32_t L = (uint32_t)(v >> half_bits) & mask, R = (uint32_t)v & mask;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const u32x4 h = philox4x32_10(u32x4{R, (uint32_t)r, 0x5045524du, 0u}, k[r], k[(r + 1) & 3]);
      const uint32_t F = h.x & mask;
      const uint32_t nl = R;
      R = L ^ F;
      L = nl;
    }
    return ((uint64_t)L << half_bits) | R;
  }
  __device__ __forceinline__ uint64_t operator()(uint64_t i) const {
    // cycle walking: the walk stays on i's cycle of a bijection, so it reaches
    // a value below n; the domain is < 4n, so a few rounds suffice on average.
    uint64_t v = round_once(i);
    for (int it = 0; v >= n && it < (1 << 20); ++it) v = round_once(v);
    return v < n ? v : i;
  }
};

__global__ void k_permute_rows(const float* __restrict__ src, int64_t n, int d, Perm p0, int64_t first, int64_t m,
                               float* __restrict__ dst) {
  const Perm p = p0.at_epoch();
  const int64_t tot = m * d;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e / d;
    const int j = (int)(e - r * d);
    const int64_t s = (int64_t)p((uint64_t)(first + r));
    dst[e] = src[s * d + j];
  }
}

// ---------------------------------------------------------------- training-data selection
// flags[i] = row i of buf [C*S, d] is all-finite
__global__ void k_finite_rows(const float* __restrict__ buf, int64_t rows, int d, int32_t* __restrict__ flags) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < rows; r += warps) {
    bool ok = true;
    for (int j = lane; j < d; j += 32) ok &= isfinite(buf[r * d + j]);
    ok = __all_sync(0xffffffffu, ok);
    if (lane == 0) flags[r] = ok ? 1 : 0;
  }
}

// block-level inclusive scan of flags -> per-block totals (pass 1), then
// exclusive offsets (pass 2), then scatter of finite row ids (pass 3)
constexpr int kScanTile = 1024;

__global__ void __launch_bounds__(kScanTile) k_scan_tiles(const int32_t* __restrict__ flags, int64_t rows,
                                                          int32_t* __restrict__ tile_tot) {
  __shared__ int32_t sh[32];
  const int64_t i = (int64_t)blockIdx.x * kScanTile + threadIdx.x;
  int v = (i < rows) ? flags[i] : 0;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int w = 0; w < kScanTile / 32; ++w) s += sh[w];
    tile_tot[blockIdx.x] = s;
  }
}

__global__ void k_scan_offsets(int32_t* __restrict__ tile_tot, int64_t n_tiles, int64_t* __restrict__ total) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int64_t s = 0;
  for (int64_t t = 0; t < n_tiles; ++t) {
    const int32_t v = tile_tot[t];
    tile_tot[t] = (int32_t)s;
    s += v;
  }
  *total = s;
}

__global__ void __launch_bounds__(kScanTile) k_scatter_finite(const int32_t* __restrict__ flags, int64_t rows,
                                                              const int32_t* __restrict__ tile_off,
                                                              int64_t* __restrict__ comp) {
  __shared__ int32_t sh[kScanTile / 32];
  const int64_t i = (int64_t)blockIdx.x * kScanTile + threadIdx.x;
  const int f = (i < rows) ? flags[i] : 0;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  // inclusive warp scan
  int v = f;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int u = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += u;
  }
  if (lane == 31) sh[w] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int k = 0; k < kScanTile / 32; ++k) {
      const int t = sh[k];
      sh[k] = s;
      s += t;
    }
  }
  __syncthreads();
  const int excl = v - f + sh[w];
  if (f) comp[tile_off[blockIdx.x] + excl] = i;
}

// out[i] = row of the compacted, per-chain-windowed data picked by index i
__global__ void k_gather_selected(const float* __restrict__ buf, int d, int C, int history, const int64_t* __restrict__ total,
                                  const int64_t* __restrict__ comp, Rng rng0, const int64_t* __restrict__ idx,
                                  int64_t n_out, float* __restrict__ out, int32_t* __restrict__ err) {
  const Rng rng = rng0.at_epoch();
  const int64_t T = *total;
  const int64_t per = (C > 0) ? T / C : 0;
  if (T % C != 0 || per == 0) {
    // the reference's reshape would fail: raise the error word and fill the
    // output with NaN, so that a caller that trains on it sees NaN losses
    // instead of stale memory
    if (blockIdx.x == 0 && threadIdx.x == 0) *err = 1;
    const int64_t tot = n_out * d;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x)
      out[e] = __int_as_float(0x7fc00000);
    return;
  }
  const int64_t hw = per < history ? per : history;
  const uint64_t N = (uint64_t)C * hw;
  const int64_t tot = n_out * d;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / d;
    const int j = (int)(e - i * d);
    uint64_t k;
    if (idx) {
      // NumPy/JAX indexing: a negative index counts from the end; what is
      // still out of range is clamped (JAX's gather clamps)
      int64_t ki = idx[i];
      if (ki < 0) ki += (int64_t)N;
      if (ki < 0) ki = 0;
      k = (uint64_t)ki;
      if (k >= N) k = N - 1;
    } else {
      const uint32_t u = rng.draw((uint64_t)i, 0, 0u, 0x53454c00u).x;
      k = ((uint64_t)u * N) >> 32;
    }
    const int64_t c = (int64_t)(k / hw), r = (int64_t)(k % hw);
    const int64_t q = c * per + (per - hw) + r;
    out[e] = buf[comp[q] * d + j];
  }
}

static int grid_ew(int64_t tot, int per_sm = 8) {
  int64_t b = (tot + 255) / 256;
  const int64_t cap = (int64_t)sm_count() * per_sm;
  if (b > cap) b = cap;
  return (int)(b < 1 ? 1 : b);
}

}  // namespace fmc

using namespace fmc;

extern "C" int fmc_adamw_workspace_size(size_t* bytes) {
  FMC_CHECK_ARG(bytes != nullptr, "bytes is NULL");
  *bytes = (kNormBlocks + 64) * sizeof(float);
  return FMC_OK;
}

extern "C" int fmc_adamw_step(float* theta, uint16_t* theta_bf16, const float* grad, float* m, float* v, int64_t n,
                              float* aux, int32_t n_aux, int32_t* count, const FmcAdamParams* p, void* ws,
                              size_t ws_bytes, void* stream) {
  FMC_CHECK_ARG(p != nullptr, "params NULL");
  FMC_CHECK_ARG(theta && grad && m && v && count, "NULL array");
  FMC_CHECK_ARG(n >= 1, "n < 1");
  FMC_CHECK_ARG(ws && ws_bytes >= (kNormBlocks + 64) * sizeof(float), "workspace too small");
  FMC_CHECK_ARG(p->max_norm > 0.f, "max_norm must be > 0");
  cudaStream_t st = (cudaStream_t)stream;
  float* part = (float*)ws;
  float* state = part + kNormBlocks;
  k_sumsq<<<kNormBlocks, 256, 0, st>>>(grad, n, part);
  FMC_LAUNCH_CHECK();
  k_norm_final<<<1, 32, 0, st>>>(part, kNormBlocks, p->max_norm, state, count);
  FMC_LAUNCH_CHECK();
  k_adamw<<<grid_ew(n, 16), 256, 0, st>>>(theta, theta_bf16, grad, m, v, n, state, count, p->lr, p->b1, p->b2, p->eps,
                                          p->weight_decay, p->max_norm, aux, n_aux);
  FMC_LAUNCH_CHECK();
  return FMC_OK;
}

extern "C" int fmc_flag_less(const float* a, float* best, int32_t* flag, void* stream) {
  FMC_CHECK_ARG(a && best && flag, "NULL pointer");
  k_flag_less<<<1, 32, 0, (cudaStream_t)stream>>>(a, best, flag);
  FMC_LAUNCH_CHECK();
  return FMC_OK;
}

extern "C" int fmc_copy_if(const int32_t* flag, const void* src, void* dst, size_t bytes, void* stream) {
  FMC_CHECK_ARG(flag && src && dst, "NULL pointer");
  FMC_CHECK_ARG(((uintptr_t)src & 15) == 0 && ((uintptr_t)dst & 15) == 0, "src/dst must be 16-byte aligned");
  if (bytes == 0) return FMC_OK;
  const int64_t n16 = (int64_t)(bytes / 16);
  const int tail = (int)(bytes % 16);
  k_copy_if<<<grid_ew(n16 > 0 ? n16 : 1), 256, 0, (cudaStream_t)stream>>>(
      flag, (const uint4*)src, (uint4*)dst, n16, (const uint8_t*)src + n16 * 16, (uint8_t*)dst + n16 * 16, tail);
  FMC_LAUNCH_CHECK();
  return FMC_OK;
}

extern "C" int fmc_column_stats_workspace_size(int64_t n, int32_t d, size_t* bytes) {
  FMC_CHECK_ARG(bytes != nullptr && n >= 2 && d >= 1, "bad arguments");
  const int dc = d < kColStatCols ? d : kColStatCols;
  *bytes = (size_t)2 * kColStatBlocks * dc * sizeof(float);
  return FMC_OK;
}

extern "C" int fmc_column_stats(const float* x, int64_t n, int32_t d, float* mean, float* var, void* ws,
                                size_t ws_bytes, void* stream) {
  FMC_CHECK_ARG(x && mean && var, "NULL pointer");
  FMC_CHECK_ARG(n >= 2 && d >= 1, "need n >= 2 rows and d >= 1");
  size_t need = 0;
  int rc = fmc_column_stats_workspace_size(n, d, &need);
  if (rc) return rc;
  FMC_CHECK_ARG(ws && ws_bytes >= need, "workspace of %zu bytes < %zu needed", ws_bytes, need);
  FMC_CHECK_ARG(((uintptr_t)ws & 15) == 0, "workspace must be 16-byte aligned");
  cudaStream_t st = (cudaStream_t)stream;
  float* part = (float*)ws;
  // column tiles of at most kColStatCols; per tile enough row blocks to cover
  // the SMs a few times over (at most kColStatBlocks, at least 64 rows each)
  for (int c0 = 0; c0 < d; c0 += kColStatCols) {
    const int dc = (d - c0 < kColStatCols) ? d - c0 : kColStatCols;
    int64_t rb = (int64_t)sm_count() * 4 * 128 / (dc < 128 ? 128 : dc);
    if (rb > kColStatBlocks) rb = kColStatBlocks;
    if (rb > (n + 63) / 64) rb = (n + 63) / 64;
    if (rb < 1) rb = 1;
    const int64_t rows_per = (n + rb - 1) / rb;
    rb = (n + rows_per - 1) / rows_per;
    dim3 grid((unsigned)rb, (unsigned)((dc + 127) / 128));
    k_colstat_partial<<<grid, 128, 0, st>>>(x + c0, n, d, dc, rows_per, part, part + rb * dc);
    FMC_LAUNCH_CHECK();
    k_colstat_final<<<(dc + 127) / 128, 128, 0, st>>>(part, part + rb * dc, (int)rb, n, dc, rows_per, mean + c0,
                                                       var + c0);
    FMC_LAUNCH_CHECK();
  }
  return FMC_OK;
}

extern "C" int fmc_permute_rows(const float* src, int64_t n, int32_t d, uint64_t seed, uint64_t counter, int64_t first,
                                int64_t m, float* dst, void* stream) {
  FMC_CHECK_ARG(src && dst, "NULL pointer");
  FMC_CHECK_ARG(n >= 1 && d >= 1 && first >= 0 && m >= 0 && first + m <= n, "bad permutation range");
  Perm p{};
  p.n = (uint64_t)n;
  int bits = 1;
  while ((1ull << (2 * bits)) < (uint64_t)n) ++bits;
  p.half_bits = bits;
  u32x4 k = philox4x32_10(u32x4{(uint32_t)counter, (uint32_t)(counter >> 32), 0x4b455953u, 0u}, (uint32_t)seed,
                          (uint32_t)(seed >> 32));
  p.k[0] = k.x; p.k[1] = k.y; p.k[2] = k.z; p.k[3] = k.w;
  p.epoch = rng_epoch();
  if (m == 0) return FMC_OK;
  k_permute_rows<<<grid_ew(m * d), 256, 0, (cudaStream_t)stream>>>(src, n, d, p, first, m, dst);
  FMC_LAUNCH_CHECK();
  return FMC_OK;
}

extern "C" int fmc_select_workspace_size(int32_t n_chains, int64_t n_steps, size_t* bytes) {
  FMC_CHECK_ARG(bytes != nullptr && n_chains >= 1 && n_steps >= 1, "bad arguments");
  // rows * 8 bytes of compacted row ids must not overflow
  FMC_CHECK_ARG(n_steps <= (INT64_MAX / 16) / n_chains, "n_chains * n_steps too large");
  const int64_t rows = (int64_t)n_chains * n_steps;
  const int64_t tiles = (rows + kScanTile - 1) / kScanTile;
  *bytes = (size_t)(rows * 4 + 256 + tiles * 4 + 256 + rows * 8 + 256 + 64);
  return FMC_OK;
}

extern "C" int fmc_select_training_data(const float* buf, int32_t n_chains, int64_t n_steps, int32_t d,
                                        int32_t history_window, int64_t n_out, uint64_t seed, uint64_t counter,
                                        const int64_t* idx, float* out, int32_t* err, void* ws, size_t ws_bytes,
                                        void* stream) {
  FMC_CHECK_ARG(buf && out && err, "NULL pointer");
  FMC_CHECK_ARG(n_chains >= 1 && n_steps >= 1 && d >= 1 && history_window >= 1 && n_out >= 1, "bad sizes");
  size_t need = 0;
  int rc = fmc_select_workspace_size(n_chains, n_steps, &need);
  if (rc) return rc;
  FMC_CHECK_ARG(ws && ws_bytes >= need, "workspace of %zu bytes < %zu needed", ws_bytes, need);
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t rows = (int64_t)n_chains * n_steps;
  const int64_t tiles = (rows + kScanTile - 1) / kScanTile;
  char* p = (char*)ws;
  int32_t* flags = (int32_t*)p;
  p += (rows * 4 + 255) / 256 * 256;
  int32_t* tile = (int32_t*)p;
  p += (tiles * 4 + 255) / 256 * 256;
  int64_t* comp = (int64_t*)p;
  p += (rows * 8 + 255) / 256 * 256;
  int64_t* total = (int64_t*)p;
  k_finite_rows<<<grid_ew(rows * 32), 256, 0, st>>>(buf, rows, d, flags);
  FMC_LAUNCH_CHECK();
  k_scan_tiles<<<(unsigned)tiles, kScanTile, 0, st>>>(flags, rows, tile);
  FMC_LAUNCH_CHECK();
  k_scan_offsets<<<1, 32, 0, st>>>(tile, tiles, total);
  FMC_LAUNCH_CHECK();
  k_scatter_finite<<<(unsigned)tiles, kScanTile, 0, st>>>(flags, rows, tile, comp);
  FMC_LAUNCH_CHECK();
  const Rng rng{(uint32_t)seed, (uint32_t)(seed >> 32), counter, rng_epoch()};
  k_gather_selected<<<grid_ew(n_out * d), 256, 0, st>>>(buf, d, n_chains, history_window, total, comp, rng, idx,
                                                        n_out, out, err);
  FMC_LAUNCH_CHECK();
  return FMC_OK;
}

namespace fmc {

// ---------------------------------------------------------------- allocation-free selection
// fmc_select_training_data_noalloc: the training-data selection for callers that
// cannot allocate device memory -- code running where cudaMalloc is off limits
// (inside another framework's allocator or a memory pool it owns, under a
// strict no-allocation policy in a serving process, or in a host callback).
// Its scratch (row flags, tile offsets, compacted row ids, the row count) lives
// in the file-scope array below, sized for at most kNoAllocSelectMaxRows =
// n_chains * n_steps rows (about 12 MiB, held by every GPU that loads the
// library until the process exits). Every call shares that array: calls that
// overlap on the GPU (different streams, or different host threads) race on
// it, so serialise them. No scratch word needs clearing between calls: each
// call writes every word it later reads.
constexpr int64_t kNoAllocSelectMaxRows = 1ll << 20;
constexpr size_t kNoAllocSelectBytes =
    (size_t)(kNoAllocSelectMaxRows * 4 + 256 + ((kNoAllocSelectMaxRows + kScanTile - 1) / kScanTile) * 4 + 256 +
             kNoAllocSelectMaxRows * 8 + 256 + 64);
static __device__ __align__(256) uint8_t g_noalloc_select_scratch[kNoAllocSelectBytes];

// the unique id of the calling thread's current context (cuCtxGetId, reached
// through the runtime's driver entry points so the library needs no -lcuda);
// 0 when no context is current yet
static int current_context_id(unsigned long long* id) {
  static PFN_cuCtxGetCurrent_v4000 get_cur = nullptr;
  static PFN_cuCtxGetId_v12000 get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_cur = (PFN_cuCtxGetCurrent_v4000)p;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = (PFN_cuCtxGetId_v12000)p;
  });
  FMC_CHECK_SUPPORTED(get_cur != nullptr && get_id != nullptr, "cuCtxGetCurrent / cuCtxGetId are unavailable");
  CUcontext ctx = nullptr;
  *id = 0;
  if (get_cur(&ctx) != CUDA_SUCCESS || ctx == nullptr) return FMC_OK;
  FMC_CHECK_SUPPORTED(get_id(ctx, id) == CUDA_SUCCESS, "cuCtxGetId failed");
  return FMC_OK;
}

static int noalloc_select_scratch(void** out) {
  // The array's name is only a host-side handle; its device address comes
  // from cudaGetSymbolAddress with the device current. The look-up is done
  // on a device's first call and cached per device, keyed by the context's
  // unique id: a context destroyed and re-created (cudaDeviceReset) reloads
  // the module, so the next call looks the address up again.
  struct Entry {
    unsigned long long ctx;
    void* addr;
  };
  static std::mutex mu;
  static Entry cache[256] = {};
  int dev = 0;
  FMC_CUDA_TRY(cudaGetDevice(&dev));
  FMC_CHECK_SUPPORTED(dev >= 0 && dev < 256, "device ordinal %d out of range", dev);
  std::lock_guard<std::mutex> lock(mu);
  unsigned long long ctx = 0;
  int rc = current_context_id(&ctx);
  if (rc) return rc;
  if (ctx == 0 || cache[dev].addr == nullptr || cache[dev].ctx != ctx) {
    void* p = nullptr;
    FMC_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_select_scratch));   // makes the primary context current
    if ((rc = current_context_id(&ctx))) return rc;
    cache[dev] = Entry{ctx, p};
  }
  *out = cache[dev].addr;
  return FMC_OK;
}

}  // namespace fmc

extern "C" int fmc_select_training_data_noalloc(const float* buf, int32_t n_chains, int64_t n_steps, int32_t d,
                                                int32_t history_window, int64_t n_out, uint64_t seed,
                                                uint64_t counter, const int64_t* idx, float* out, int32_t* err,
                                                void* stream) {
  FMC_CHECK_ARG(n_chains >= 1 && n_steps >= 1, "bad sizes");
  // compare before multiplying, so that no product can overflow
  FMC_CHECK_ARG(n_steps <= fmc::kNoAllocSelectMaxRows / n_chains,
                "n_chains * n_steps exceeds the %lld rows the static scratch of "
                "fmc_select_training_data_noalloc holds; use fmc_select_training_data with a workspace",
                (long long)fmc::kNoAllocSelectMaxRows);
  const int64_t rows = (int64_t)n_chains * n_steps;
  FMC_CHECK_ARG(rows <= fmc::kNoAllocSelectMaxRows,
                "n_chains * n_steps = %lld rows exceeds the %lld rows the static scratch of "
                "fmc_select_training_data_noalloc holds; use fmc_select_training_data with a workspace",
                (long long)rows, (long long)fmc::kNoAllocSelectMaxRows);
  void* scratch = nullptr;
  int rc = fmc::noalloc_select_scratch(&scratch);
  if (rc) return rc;
  return fmc_select_training_data(buf, n_chains, n_steps, d, history_window, n_out, seed, counter, idx, out, err,
                                  scratch, fmc::kNoAllocSelectBytes, stream);
}
