// tempering.cu -- parallel tempering (strategy/parallel_tempering.py of flowMC).
//
// One ParallelTempering call is three launches:
//  1. the tempered local steps: K1 over the n_chains * n_temps rows of the
//     (chain, temperature) ensemble, row c at inverse temperature
//     1 / temps[c % n_temps], no per-step rows stored (the reference keeps
//     only the last state of each tempered chain, parallel_tempering.py:205-248);
//  2. the exchange sweep (k_pt_exchange): per chain, the untempered
//     log-density of every temperature's position, then the sequential
//     adjacent-pair swaps (parallel_tempering.py:291-398), then the positions
//     written out in swapped order -- the T=1 row to the chain position, the
//     rest to the tempered-positions buffer;
//  3. the temperature adaptation (k_pt_adapt, parallel_tempering.py:400-436)
//     from exact integer swap counts per adjacent pair.
#include "local_steps.cuh"

namespace fmc {

constexpr int kMaxTemps = 64;

struct ExchangeArgs {
  FmcTarget tgt;
  const float* x;       // [C * T, d] positions after the tempered steps
  int32_t C, T, d;
  const float* temps;   // [T]
  Rng rng;
  const float* unif;    // [C, T - 1] explicit uniforms, or NULL (in-kernel Philox)
  float* out_first;     // [C, d] temperature-1 position after the sweep
  float* out_rest;      // [C, T - 1, d] tempered positions after the sweep, or NULL
  float* out_logp;      // [C, T] untempered log-density after the sweep, or NULL
  float* out_acc;       // [C, T - 1] swap flags (1 / 0), or NULL
  int32_t* acc_pairs;   // [T - 1] accepted swaps per adjacent pair (added to)
  int64_t C_pad;
};

template <int G, int V>
__device__ __forceinline__ void load_row(const float* __restrict__ row, float (&x)[V], int gl, int d) {
#pragma unroll
  for (int v = 0; v < V; ++v) {
    const int j = gl * V + v;
    x[v] = (j < d) ? __ldg(row + j) : 0.f;
  }
}

// One lane group per chain. The group evaluates log L at each of the chain's
// T positions, lane 0 of the group runs the swap sweep in shared memory (the
// sweep is sequential: a swap at pair i moves the position pair i + 1
// compares), and the group then copies the rows out in their new order.
template <int TGT, int G, int V>
__global__ void __launch_bounds__(256) k_pt_exchange(const ExchangeArgs a) {
  extern __shared__ float smem[];
  const int gl = threadIdx.x % G;
  const int gpb = blockDim.x / G, gib = threadIdx.x / G;
  const int T = a.T, d = a.d;
  float* stage = (TGT == FMC_TARGET_DENSE_GAUSSIAN) ? smem + gib * d : nullptr;
  float* tail = smem + ((TGT == FMC_TARGET_DENSE_GAUSSIAN) ? gpb * d : 0);
  int* cnt = reinterpret_cast<int*>(tail);                  // [kMaxTemps]
  float* Ls = tail + kMaxTemps + gib * T;                    // this group's log-densities
  int* perm = reinterpret_cast<int*>(tail + kMaxTemps + gpb * T) + gib * T;
  for (int i = threadIdx.x; i < kMaxTemps; i += blockDim.x) cnt[i] = 0;
  const Rng rng = a.rng.at_epoch();
  __syncthreads();

  for (int64_t c = blockIdx.x * (int64_t)gpb + gib; c < a.C_pad; c += (int64_t)gridDim.x * gpb) {
    const bool active = c < a.C;
    const int64_t cc = active ? c : 0;
    const float* xc = a.x + cc * T * d;
    for (int t = 0; t < T; ++t) {
      float xv[V], gv[V];
      load_row<G, V>(xc + (int64_t)t * d, xv, gl, d);
      const float l = target_eval<TGT, G, V, false>(a.tgt, xv, gv, gl, stage);
      if (gl == 0) {
        Ls[t] = l;
        perm[t] = t;
      }
    }
    __syncwarp();
    if (gl == 0) {
      float inv_lo = __fdiv_rn(1.f, __ldg(a.temps));
      for (int i = 0; i + 1 < T; ++i) {
        const float inv_hi = __fdiv_rn(1.f, __ldg(a.temps + i + 1));
        // (1/T[i+1] - 1/T[i]) * (lp[i] - lp[i+1])   (parallel_tempering.py:297-299)
        const float ratio = (inv_hi - inv_lo) * (Ls[i] - Ls[i + 1]);
        float u;
        if (a.unif) {
          u = __ldg(a.unif + cc * (T - 1) + i);
        } else {
          const u32x4 r = rng.draw((uint64_t)cc, (uint64_t)i, 0u, RNG_TAG_PT_EXCHANGE);
          u = u32_to_unit(r.x);
        }
        const bool acc = logf(u) < ratio;
        if (acc) {
          const float tl = Ls[i];
          Ls[i] = Ls[i + 1];
          Ls[i + 1] = tl;
          const int tp = perm[i];
          perm[i] = perm[i + 1];
          perm[i + 1] = tp;
        }
        if (active) {
          if (a.out_acc) a.out_acc[cc * (T - 1) + i] = acc ? 1.f : 0.f;
          if (acc) atomicAdd(&cnt[i], 1);
        }
        inv_lo = inv_hi;
      }
    }
    __syncwarp();
    for (int t = 0; t < T; ++t) {
      float* dst = (t == 0) ? a.out_first + cc * d
                   : (a.out_rest ? a.out_rest + (cc * (T - 1) + (t - 1)) * d : nullptr);
      if (dst != nullptr) {
        float xv[V];
        load_row<G, V>(xc + (int64_t)perm[t] * d, xv, gl, d);
        if (active) {
#pragma unroll
          for (int v = 0; v < V; ++v) {
            const int j = gl * V + v;
            if (j < d) dst[j] = xv[v];
          }
        }
      }
      if (a.out_logp && active && gl == 0) a.out_logp[cc * T + t] = Ls[t];
    }
    __syncwarp();   // the next chain reuses Ls / perm
  }
  __syncthreads();
  for (int i = threadIdx.x; i + 1 < T; i += blockDim.x)
    if (cnt[i]) atomicAdd(a.acc_pairs + i, cnt[i]);
}

// _adapt_temperature (parallel_tempering.py:400-436): acceptance rate per
// adjacent pair = swaps / n_chains, damping = (100 / n_chains) * (rate[i] -
// rate[i+1]), T'[i] = T'[i-1] + (T[i] - T[i-1]) * exp(damping[i-1]) for
// 0 < i < n_temps - 1 (the end temperatures stay). One thread: n_temps <= 64.
__global__ void k_pt_adapt(const float* temps, const int32_t* acc_pairs, int32_t C, int32_t T, float* out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  float old[kMaxTemps], nw[kMaxTemps];
  for (int i = 0; i < T; ++i) old[i] = temps[i];
  // the reference's Python-float scale, rounded once to fp32
  const float scale = (float)(100.0 / (double)C);
  nw[0] = old[0];
  for (int i = 1; i + 1 < T; ++i) {
    const float r0 = __fdiv_rn((float)acc_pairs[i - 1], (float)C);
    const float r1 = __fdiv_rn((float)acc_pairs[i], (float)C);
    nw[i] = nw[i - 1] + (old[i] - old[i - 1]) * expf(scale * (r0 - r1));
  }
  if (T > 1) nw[T - 1] = old[T - 1];
  for (int i = 0; i < T; ++i) out[i] = nw[i];
}

template <int TGT, int G, int V>
static int launch_exchange_t(const ExchangeArgs& a0, cudaStream_t st) {
  ExchangeArgs a = a0;
  const int threads = 256, gpb = threads / G, gpw = 32 / G;
  a.C_pad = ((int64_t)a.C + gpw - 1) / gpw * gpw;
  size_t smem = ((TGT == FMC_TARGET_DENSE_GAUSSIAN) ? (size_t)gpb * a.d : 0) + kMaxTemps + (size_t)2 * gpb * a.T;
  smem *= sizeof(float);
  auto kern = k_pt_exchange<TGT, G, V>;
  if (smem > 48 * 1024) FMC_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  FMC_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem));
  if (per_sm < 1) per_sm = 1;
  const int64_t need = (a.C_pad + gpb - 1) / gpb;
  const int64_t cap = (int64_t)sm_count() * per_sm;
  kern<<<(int)(need < cap ? need : cap), threads, smem, st>>>(a);
  FMC_LAUNCH_CHECK();
  return FMC_OK;
}

template <int TGT>
static int launch_exchange_tgt(const ExchangeArgs& a, cudaStream_t st) {
  const Shape sh = default_shape(a.d);
#define FMC_PT_CASE(g, v) \
  if (sh.G == g && sh.V == v) return launch_exchange_t<TGT, g, v>(a, st);
  FMC_PT_CASE(4, 1) FMC_PT_CASE(8, 1) FMC_PT_CASE(8, 2) FMC_PT_CASE(8, 4)
  FMC_PT_CASE(16, 4) FMC_PT_CASE(32, 4) FMC_PT_CASE(32, 8)
#undef FMC_PT_CASE
  set_error("no exchange shape for n_dim=%d", a.d);
  return FMC_ERR_UNSUPPORTED;
}

}  // namespace fmc

using namespace fmc;

extern "C" int fmc_pt_local_steps(const FmcTarget* target, const FmcLocalParams* params, const float* x0,
                                  int32_t n_chains, int32_t n_temps, const float* temperatures,
                                  const float* prior_mean, const float* prior_inv_var, float prior_const,
                                  int32_t n_steps, uint64_t seed, uint64_t counter, const float* noise,
                                  const float* unif, float* x_last, float* lp_last, float* acc_count,
                                  void* stream) {
  int rc = check_target(target);
  if (rc) return rc;
  FMC_CHECK_ARG(params != nullptr, "params is NULL");
  FMC_CHECK_ARG(params->kind >= 0 && params->kind <= FMC_KERNEL_GRW, "unknown kernel kind %d", params->kind);
  FMC_CHECK_ARG(params->kind != FMC_KERNEL_HMC || params->n_leapfrog >= 0, "n_leapfrog < 0");
  FMC_CHECK_ARG(n_chains >= 0, "n_chains=%d < 0", n_chains);
  FMC_CHECK_ARG(n_temps >= 1 && n_temps <= kMaxTemps, "n_temps=%d outside [1, %d]", n_temps, kMaxTemps);
  FMC_CHECK_ARG((int64_t)n_chains * n_temps <= INT32_MAX, "n_chains * n_temps exceeds 2^31 - 1");
  FMC_CHECK_ARG(n_steps >= 1, "n_steps=%d < 1", n_steps);
  FMC_CHECK_ARG((prior_mean == nullptr) == (prior_inv_var == nullptr),
                "a diagonal Gaussian prior needs both its mean and its inverse variances");
  if (n_chains == 0) return FMC_OK;
  FMC_CHECK_ARG(x0 && temperatures && x_last && lp_last, "NULL array argument");
  if (target->kind == FMC_TARGET_DENSE_GAUSSIAN)
    FMC_CHECK_SUPPORTED(target->n_dim <= 128, "dense Gaussian group kernel supports n_dim <= 128");

  LocalArgs a{};
  a.tgt = *target;
  a.n_leapfrog = params->n_leapfrog;
  a.step = params->step_size;
  a.mscale = params->momentum_scale;
  a.mcol = params->metric_colsum;
  a.mchol = params->momentum_chol;
  a.x0 = x0;
  a.lp0 = nullptr;   // the tempered log-density is evaluated at x0 (parallel_tempering.py:236-238)
  a.C = n_chains * n_temps;
  a.d = target->n_dim;
  a.S = n_steps;
  a.thin = 1;
  a.rng = Rng{(uint32_t)seed, (uint32_t)(seed >> 32), counter, rng_epoch()};
  a.noise = noise;
  a.unif = unif;
  a.buf_len = 1;
  a.x_last = x_last;
  a.lp_last = lp_last;
  a.temps = temperatures;
  a.n_temps = n_temps;
  a.prior_mean = prior_mean;
  a.prior_iv = prior_inv_var;
  a.prior_const = prior_const;
  a.acc_count = acc_count;
  return dispatch_local(a, params, (cudaStream_t)stream);
}

extern "C" int fmc_pt_exchange(const FmcTarget* target, const float* x, int32_t n_chains, int32_t n_temps,
                               const float* temperatures, uint64_t seed, uint64_t counter, const float* unif,
                               float* out_first, float* out_rest, float* out_logp, float* out_acc,
                               int32_t* acc_pairs, void* stream) {
  int rc = check_target(target);
  if (rc) return rc;
  FMC_CHECK_ARG(n_chains >= 0, "n_chains=%d < 0", n_chains);
  FMC_CHECK_ARG(n_temps >= 1 && n_temps <= kMaxTemps, "n_temps=%d outside [1, %d]", n_temps, kMaxTemps);
  FMC_CHECK_ARG(acc_pairs != nullptr || n_temps == 1, "acc_pairs is NULL");
  cudaStream_t st = (cudaStream_t)stream;
  if (n_temps > 1) FMC_CUDA_TRY(cudaMemsetAsync(acc_pairs, 0, sizeof(int32_t) * (n_temps - 1), st));
  if (n_chains == 0) return FMC_OK;
  FMC_CHECK_ARG(x && temperatures && out_first, "NULL array argument");
  if (target->kind == FMC_TARGET_DENSE_GAUSSIAN)
    FMC_CHECK_SUPPORTED(target->n_dim <= 128, "dense Gaussian group kernel supports n_dim <= 128");
  ExchangeArgs a{};
  a.tgt = *target;
  a.x = x;
  a.C = n_chains;
  a.T = n_temps;
  a.d = target->n_dim;
  a.temps = temperatures;
  a.rng = Rng{(uint32_t)seed, (uint32_t)(seed >> 32), counter, rng_epoch()};
  a.unif = unif;
  a.out_first = out_first;
  a.out_rest = out_rest;
  a.out_logp = out_logp;
  a.out_acc = out_acc;
  a.acc_pairs = acc_pairs;
  switch (target->kind) {
    case FMC_TARGET_DIAG_GAUSSIAN: return launch_exchange_tgt<FMC_TARGET_DIAG_GAUSSIAN>(a, st);
    case FMC_TARGET_DUAL_MOON: return launch_exchange_tgt<FMC_TARGET_DUAL_MOON>(a, st);
    case FMC_TARGET_GAUSS_MIXTURE: return launch_exchange_tgt<FMC_TARGET_GAUSS_MIXTURE>(a, st);
    case FMC_TARGET_ROSENBROCK: return launch_exchange_tgt<FMC_TARGET_ROSENBROCK>(a, st);
    default: return launch_exchange_tgt<FMC_TARGET_DENSE_GAUSSIAN>(a, st);
  }
}

extern "C" int fmc_pt_adapt_temperatures(const float* temperatures, const int32_t* acc_pairs, int32_t n_chains,
                                         int32_t n_temps, float* out_temperatures, void* stream) {
  FMC_CHECK_ARG(n_chains >= 1, "n_chains=%d < 1", n_chains);
  FMC_CHECK_ARG(n_temps >= 1 && n_temps <= kMaxTemps, "n_temps=%d outside [1, %d]", n_temps, kMaxTemps);
  FMC_CHECK_ARG(temperatures && out_temperatures && (acc_pairs || n_temps == 1), "NULL array argument");
  k_pt_adapt<<<1, 32, 0, (cudaStream_t)stream>>>(temperatures, acc_pairs, n_chains, n_temps, out_temperatures);
  FMC_LAUNCH_CHECK();
  return FMC_OK;
}
