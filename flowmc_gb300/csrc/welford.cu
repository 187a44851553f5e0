// welford.cu -- streaming FP64 moments and batch-means ESS of chain rows,
// accumulated on the device while the sampler runs (no counterpart in the
// reference, whose tutorials compute diagnostics afterwards with arviz).
//
// State (caller-owned, fmc_welford_state_size bytes, 8-byte aligned):
//   int64 n_seen  draws per chain accumulated so far
//   int64 batch   draws per batch of the batch-means estimator
//   then five float64 arrays [n_chains][n_dim]:
//     mean, m2          Welford's running mean and sum of squared deviations
//                       (Welford, Technometrics 4, 1962) of each chain's draws
//     bsum              the sum of the current, incomplete batch
//     bmean, bm2        Welford over the chain's completed batch means
//
// fmc_welford_ess_update folds rows [start, start + n_steps) of every chain of
// a chain buffer [n_chains, buf_len, n_dim] (float32) into the state: one
// thread per (chain, coordinate), consecutive threads on consecutive
// coordinates, so each row is read coalesced; the draw count lives in the
// state, so a captured CUDA graph can replay the update. fmc_welford_ess_finalize
// merges the chains per coordinate in a fixed order (Chan, Golub & LeVeque,
// 1979): grand mean, the variance of all draws, the within-chain variance W,
// R-hat = sqrt(((n-1)/n W + B/n) / W) (Gelman & Rubin 1992), and the
// multi-chain batch-means ESS = N var / (b var_bm): N draws, b the batch
// size, var_bm the variance of all completed batch means (Flegal & Jones,
// "Batch means and spectral variance estimators in MCMC", Ann. Stat. 2010).
#include "common.cuh"

namespace fmc {

struct WelfordView {
  int64_t* hdr;   // n_seen, batch
  double *mean, *m2, *bsum, *bmean, *bm2;
};

static WelfordView welford_view(double* state, int64_t n_chains, int n_dim) {
  const int64_t cd = n_chains * n_dim;
  WelfordView v;
  v.hdr = reinterpret_cast<int64_t*>(state);
  v.mean = state + 2;
  v.m2 = v.mean + cd;
  v.bsum = v.m2 + cd;
  v.bmean = v.bsum + cd;
  v.bm2 = v.bmean + cd;
  return v;
}

__global__ void k_welford_reset(WelfordView v, int64_t cd, int64_t batch) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < cd; i += (int64_t)gridDim.x * blockDim.x) {
    v.mean[i] = 0.0;
    v.m2[i] = 0.0;
    v.bsum[i] = 0.0;
    v.bmean[i] = 0.0;
    v.bm2[i] = 0.0;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    v.hdr[0] = 0;
    v.hdr[1] = batch;
  }
}

// steps per launch of the update kernel: the block's table of 1 / n holds
// this many float64 values (the host splits longer updates)
constexpr int kWelfordSteps = 2048;

__global__ void k_welford_update(WelfordView v, const float* __restrict__ buf, int64_t n_chains, int64_t buf_len,
                                 int n_dim, int64_t start, int n_steps) {
  __shared__ double inv_n[kWelfordSteps];   // 1 / n of every step (one FP64 division per step per block)
  const int64_t n0 = v.hdr[0], batch = v.hdr[1];
  for (int s = threadIdx.x; s < n_steps; s += blockDim.x) inv_n[s] = 1.0 / (double)(n0 + s + 1);
  __syncthreads();
  const int64_t cd = n_chains * n_dim;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < cd; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = i / n_dim;
    const int j = (int)(i - c * n_dim);
    double mean = v.mean[i], m2 = v.m2[i], bsum = v.bsum[i], bmean = v.bmean[i], bm2 = v.bm2[i];
    const float* row = buf + (c * buf_len + start) * n_dim + j;
    int64_t in_batch = n0 % batch;   // draws of the current batch so far
    for (int s = 0; s < n_steps; ++s) {
      const double x = (double)__ldg(row + (int64_t)s * n_dim);
      const double delta = x - mean;
      mean += delta * inv_n[s];
      m2 += delta * (x - mean);
      bsum += x;
      if (++in_batch == batch) {
        in_batch = 0;
        const double bm = bsum / (double)batch;
        const int64_t k = (n0 + s + 1) / batch;
        const double bd = bm - bmean;
        bmean += bd / (double)k;
        bm2 += bd * (bm - bmean);
        bsum = 0.0;
      }
    }
    v.mean[i] = mean;
    v.m2[i] = m2;
    v.bsum[i] = bsum;
    v.bmean[i] = bmean;
    v.bm2[i] = bm2;
  }
}

__global__ void k_welford_advance(int64_t* hdr, int n_steps) { hdr[0] += n_steps; }

// one block per coordinate; threads take chains c = tid, tid + blockDim, ...
// and the partial sums are combined by a fixed-order tree
constexpr int kFinThreads = 256;

__device__ __forceinline__ double block_sum(double v, double* sh) {
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int o = kFinThreads / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  const double r = sh[0];
  __syncthreads();
  return r;
}

__global__ void __launch_bounds__(kFinThreads) k_welford_finalize(WelfordView v, int64_t n_chains, int n_dim,
                                                                  double* __restrict__ mean_out,
                                                                  double* __restrict__ var_out,
                                                                  double* __restrict__ ess_out,
                                                                  double* __restrict__ rhat_out) {
  __shared__ double sh[kFinThreads];
  const int j = blockIdx.x;
  const int64_t n = v.hdr[0], batch = v.hdr[1], k = n / batch;
  const double C = (double)n_chains;
  double s_mean = 0.0, s_m2 = 0.0, s_bmean = 0.0, s_bm2 = 0.0;
  for (int64_t c = threadIdx.x; c < n_chains; c += kFinThreads) {
    const int64_t i = c * n_dim + j;
    s_mean += v.mean[i];
    s_m2 += v.m2[i];
    s_bmean += v.bmean[i];
    s_bm2 += v.bm2[i];
  }
  const double mu = block_sum(s_mean, sh) / C;
  const double sum_m2 = block_sum(s_m2, sh);
  const double mub = block_sum(s_bmean, sh) / C;
  const double sum_bm2 = block_sum(s_bm2, sh);
  double s_dev = 0.0, s_bdev = 0.0;
  for (int64_t c = threadIdx.x; c < n_chains; c += kFinThreads) {
    const int64_t i = c * n_dim + j;
    const double a = v.mean[i] - mu, b = v.bmean[i] - mub;
    s_dev += a * a;
    s_bdev += b * b;
  }
  const double dev = block_sum(s_dev, sh);
  const double bdev = block_sum(s_bdev, sh);
  if (threadIdx.x == 0) {
    const double N = C * (double)n;
    const double var = (n > 0 && N > 1.0) ? (sum_m2 + (double)n * dev) / (N - 1.0) : 0.0;
    mean_out[j] = mu;
    var_out[j] = var;
    // R-hat from the within-chain variance W and the between-chain B / n
    const double W = n > 1 ? sum_m2 / (C * (double)(n - 1)) : 0.0;
    const double B_n = n_chains > 1 ? dev / (C - 1.0) : 0.0;
    rhat_out[j] = (W > 0.0 && n > 0) ? sqrt((((double)(n - 1) / (double)n) * W + B_n) / W) : NAN;
    // batch means: variance of all C * k completed batch means
    const double Kb = C * (double)k;
    const double var_bm = Kb > 1.0 ? (sum_bm2 + (double)k * bdev) / (Kb - 1.0) : 0.0;
    double ess = NAN;
    if (Kb > 1.0 && var > 0.0) {
      const double tau = (double)batch * var_bm / var;   // integrated autocorrelation time
      ess = tau > 0.0 ? N / tau : N;
      if (ess > N) ess = N;
    }
    ess_out[j] = ess;
  }
}

}  // namespace fmc

using namespace fmc;

extern "C" int fmc_welford_state_size(int32_t n_chains, int32_t n_dim, size_t* bytes) {
  FMC_CHECK_ARG(bytes != nullptr && n_chains >= 1 && n_dim >= 1, "bad arguments");
  *bytes = (size_t)(2 + 5 * (int64_t)n_chains * n_dim) * sizeof(double);
  return FMC_OK;
}

static int grid_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  const int64_t cap = (int64_t)sm_count() * 8;
  if (b > cap) b = cap;
  return (int)(b < 1 ? 1 : b);
}

extern "C" int fmc_welford_reset(double* state, int32_t n_chains, int32_t n_dim, int32_t batch, void* stream) {
  FMC_CHECK_ARG(state != nullptr && n_chains >= 1 && n_dim >= 1, "bad arguments");
  FMC_CHECK_ARG(batch >= 1, "batch must be >= 1");
  FMC_CHECK_ARG(((uintptr_t)state & 7) == 0, "state must be 8-byte aligned");
  const int64_t cd = (int64_t)n_chains * n_dim;
  k_welford_reset<<<grid_for(cd), 256, 0, (cudaStream_t)stream>>>(welford_view(state, n_chains, n_dim), cd, batch);
  FMC_LAUNCH_CHECK();
  return FMC_OK;
}

extern "C" int fmc_welford_ess_update(const float* buf, int32_t n_chains, int64_t buf_len, int32_t n_dim,
                                      int64_t start, int32_t n_steps, double* state, void* stream) {
  FMC_CHECK_ARG(buf != nullptr && state != nullptr, "NULL pointer");
  FMC_CHECK_ARG(n_chains >= 1 && n_dim >= 1 && n_steps >= 0, "bad sizes");
  FMC_CHECK_ARG(start >= 0 && start + n_steps <= buf_len, "rows [%lld, %lld) outside a buffer of %lld rows",
                (long long)start, (long long)(start + n_steps), (long long)buf_len);
  FMC_CHECK_ARG(((uintptr_t)state & 7) == 0, "state must be 8-byte aligned");
  if (n_steps == 0) return FMC_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t cd = (int64_t)n_chains * n_dim;
  const WelfordView v = welford_view(state, n_chains, n_dim);
  for (int s0 = 0; s0 < n_steps; s0 += kWelfordSteps) {
    const int ns = n_steps - s0 < kWelfordSteps ? n_steps - s0 : kWelfordSteps;
    k_welford_update<<<grid_for(cd), 256, 0, st>>>(v, buf, n_chains, buf_len, n_dim, start + s0, ns);
    FMC_LAUNCH_CHECK();
    k_welford_advance<<<1, 1, 0, st>>>(v.hdr, ns);
    FMC_LAUNCH_CHECK();
  }
  return FMC_OK;
}

extern "C" int fmc_welford_ess_finalize(const double* state, int32_t n_chains, int32_t n_dim, double* mean,
                                        double* var, double* ess, double* rhat, void* stream) {
  FMC_CHECK_ARG(state && mean && var && ess && rhat, "NULL pointer");
  FMC_CHECK_ARG(n_chains >= 1 && n_dim >= 1, "bad sizes");
  const WelfordView v = welford_view(const_cast<double*>(state), n_chains, n_dim);
  k_welford_finalize<<<n_dim, kFinThreads, 0, (cudaStream_t)stream>>>(v, n_chains, n_dim, mean, var, ess, rhat);
  FMC_LAUNCH_CHECK();
  return FMC_OK;
}
