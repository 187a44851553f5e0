// optimization.cu -- AdamOptimization (strategy/optimization.py of flowMC):
// n_steps of Adam on -log p(x) for every chain in one persistent launch.
//
// Per chain and step (optimization.py:117-129): the objective's gradient
// -grad log p(x) is multiplied by (1 + xi * noise_level) with one standard
// normal xi per chain-step, then optax.adam (b1 = 0.9, b2 = 0.999, eps = 1e-8,
// eps_root = 0: optax's defaults) and the projection onto the box
// [lower, upper]. A lane group owns a chain: position, first and second
// moments stay in registers for the whole run; the target's value and
// gradient are the fused device targets of the local-step kernel.
#include "local_steps.cuh"

namespace fmc {

struct AdamOptArgs {
  FmcTarget tgt;
  const float* x0;
  int32_t C, d, S;
  float lr, noise_level;
  const float* lower;   // [d] or NULL (no bound)
  const float* upper;
  Rng rng;
  const float* noise;   // [C, S] explicit normals or NULL (Philox)
  float* x_out;
  float* lp_out;        // [C] log p at the result, or NULL
  int64_t C_pad;
};

constexpr float kAdamB1 = 0.9f, kAdamB2 = 0.999f, kAdamEps = 1e-8f;

template <int TGT, int G, int V>
__global__ void __launch_bounds__(256) k_adam_optimize(const AdamOptArgs a) {
  extern __shared__ float smem[];
  const int gl = threadIdx.x % G;
  const int gpb = blockDim.x / G, gib = threadIdx.x / G;
  const int d = a.d;
  float* stage = (TGT == FMC_TARGET_DENSE_GAUSSIAN) ? smem + gib * d : nullptr;
  const Rng rng = a.rng.at_epoch();
  float lo[V], hi[V];
#pragma unroll
  for (int v = 0; v < V; ++v) {
    const int j = gl * V + v;
    lo[v] = (a.lower && j < d) ? __ldg(a.lower + j) : -INFINITY;
    hi[v] = (a.upper && j < d) ? __ldg(a.upper + j) : INFINITY;
  }
  for (int64_t c = blockIdx.x * (int64_t)gpb + gib; c < a.C_pad; c += (int64_t)gridDim.x * gpb) {
    const bool active = c < a.C;
    const int64_t cc = active ? c : 0;
    float x[V], m[V], s2[V], g[V];
#pragma unroll
    for (int v = 0; v < V; ++v) {
      const int j = gl * V + v;
      x[v] = (j < d) ? __ldg(a.x0 + cc * d + j) : 0.f;
      m[v] = 0.f;
      s2[v] = 0.f;
    }
    for (int s = 0; s < a.S; ++s) {
      target_eval<TGT, G, V, true>(a.tgt, x, g, gl, stage);
      float xi;
      if (a.noise) {
        xi = __ldg(a.noise + cc * a.S + s);
      } else {
        const u32x4 r = rng.draw((uint64_t)cc, (uint64_t)s, 0u, RNG_TAG_ADAM_NOISE);
        float z1;
        box_muller(r.x, r.y, xi, z1);
      }
      const float f = 1.f + xi * a.noise_level;
      // bias corrections 1 - b^t with t = s + 1 (optax's decay ** count)
      const float t = (float)(s + 1);
      const float bc1 = 1.f - powf(kAdamB1, t), bc2 = 1.f - powf(kAdamB2, t);
#pragma unroll
      for (int v = 0; v < V; ++v) {
        const float gr = -g[v] * f;                                 // grad of -log p, noised
        m[v] = (1.f - kAdamB1) * gr + kAdamB1 * m[v];
        s2[v] = (1.f - kAdamB2) * (gr * gr) + kAdamB2 * s2[v];
        const float upd = (m[v] / bc1) / (sqrtf(s2[v] / bc2) + kAdamEps);
        // apply, then project (jnp.clip: a NaN position stays NaN)
        const float xn = x[v] + upd * (-a.lr);
        x[v] = xn < lo[v] ? lo[v] : (xn > hi[v] ? hi[v] : xn);
      }
    }
    const float lp = target_eval<TGT, G, V, false>(a.tgt, x, g, gl, stage);
    if (active) {
#pragma unroll
      for (int v = 0; v < V; ++v) {
        const int j = gl * V + v;
        if (j < d) a.x_out[cc * d + j] = x[v];
      }
      if (a.lp_out && gl == 0) a.lp_out[cc] = lp;
    }
  }
}

template <int TGT, int G, int V>
static int launch_adam_t(const AdamOptArgs& a0, cudaStream_t st) {
  AdamOptArgs a = a0;
  const int threads = 256, gpb = threads / G, gpw = 32 / G;
  a.C_pad = ((int64_t)a.C + gpw - 1) / gpw * gpw;
  const size_t smem = (TGT == FMC_TARGET_DENSE_GAUSSIAN) ? (size_t)gpb * a.d * sizeof(float) : 0;
  auto kern = k_adam_optimize<TGT, G, V>;
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
static int launch_adam_tgt(const AdamOptArgs& a, cudaStream_t st) {
  const Shape sh = default_shape(a.d);
#define FMC_ADAM_CASE(g, v) \
  if (sh.G == g && sh.V == v) return launch_adam_t<TGT, g, v>(a, st);
  FMC_ADAM_CASE(4, 1) FMC_ADAM_CASE(8, 1) FMC_ADAM_CASE(8, 2) FMC_ADAM_CASE(8, 4)
  FMC_ADAM_CASE(16, 4) FMC_ADAM_CASE(32, 4) FMC_ADAM_CASE(32, 8)
#undef FMC_ADAM_CASE
  set_error("no optimisation shape for n_dim=%d", a.d);
  return FMC_ERR_UNSUPPORTED;
}

}  // namespace fmc

using namespace fmc;

extern "C" int fmc_adam_optimize(const FmcTarget* target, const float* x0, int32_t n_chains, int32_t n_steps,
                                 float learning_rate, float noise_level, const float* lower, const float* upper,
                                 uint64_t seed, uint64_t counter, const float* noise, float* x_out, float* lp_out,
                                 void* stream) {
  int rc = check_target(target);
  if (rc) return rc;
  FMC_CHECK_ARG(n_chains >= 0, "n_chains=%d < 0", n_chains);
  FMC_CHECK_ARG(n_steps >= 0, "n_steps=%d < 0", n_steps);
  if (n_chains == 0) return FMC_OK;
  FMC_CHECK_ARG(x0 && x_out, "NULL array argument");
  if (target->kind == FMC_TARGET_DENSE_GAUSSIAN)
    FMC_CHECK_SUPPORTED(target->n_dim <= 128, "dense Gaussian group kernel supports n_dim <= 128");
  AdamOptArgs a{};
  a.tgt = *target;
  a.x0 = x0;
  a.C = n_chains;
  a.d = target->n_dim;
  a.S = n_steps;
  a.lr = learning_rate;
  a.noise_level = noise_level;
  a.lower = lower;
  a.upper = upper;
  a.rng = Rng{(uint32_t)seed, (uint32_t)(seed >> 32), counter, rng_epoch()};
  a.noise = noise;
  a.x_out = x_out;
  a.lp_out = lp_out;
  cudaStream_t st = (cudaStream_t)stream;
  switch (target->kind) {
    case FMC_TARGET_DIAG_GAUSSIAN: return launch_adam_tgt<FMC_TARGET_DIAG_GAUSSIAN>(a, st);
    case FMC_TARGET_DUAL_MOON: return launch_adam_tgt<FMC_TARGET_DUAL_MOON>(a, st);
    case FMC_TARGET_GAUSS_MIXTURE: return launch_adam_tgt<FMC_TARGET_GAUSS_MIXTURE>(a, st);
    case FMC_TARGET_ROSENBROCK: return launch_adam_tgt<FMC_TARGET_ROSENBROCK>(a, st);
    default: return launch_adam_tgt<FMC_TARGET_DENSE_GAUSSIAN>(a, st);
  }
}
