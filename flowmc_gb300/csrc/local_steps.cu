// local_steps.cu -- C entry points of K1 and the batch target evaluation.
#include "local_steps.cuh"

namespace fmc {

int check_target(const FmcTarget* t) {
  FMC_CHECK_ARG(t != nullptr, "target is NULL");
  FMC_CHECK_ARG(t->n_dim >= 1 && t->n_dim <= 256, "n_dim=%d outside [1, 256]", t->n_dim);
  FMC_CHECK_ARG(t->kind >= 0 && t->kind <= FMC_TARGET_DENSE_GAUSSIAN, "unknown target kind %d", t->kind);
  if (t->kind == FMC_TARGET_GAUSS_MIXTURE) {
    FMC_CHECK_ARG(t->n_comp >= 1 && t->n_comp <= kMaxMixtureComponents,
                  "mixture n_comp=%d outside [1, %d]", t->n_comp, kMaxMixtureComponents);
    FMC_CHECK_ARG(t->mean != nullptr, "mixture needs means");
  }
  if (t->kind == FMC_TARGET_DENSE_GAUSSIAN) FMC_CHECK_ARG(t->precision != nullptr, "dense Gaussian needs a precision matrix");
  if (t->kind == FMC_TARGET_DUAL_MOON) FMC_CHECK_ARG(t->scalars[1] != 0.f && t->scalars[3] != 0.f, "dual moon scales must be non-zero");
  if (t->kind == FMC_TARGET_ROSENBROCK) FMC_CHECK_ARG(t->scalars[0] != 0.f, "Rosenbrock divisor must be non-zero");
  return FMC_OK;
}

int dispatch_local(const LocalArgs& a, const FmcLocalParams* params, cudaStream_t st) {
  Shape sh = default_shape(a.d);
  if (params->lanes_per_chain > 0) {
    const int G = params->lanes_per_chain;
    FMC_CHECK_SUPPORTED(G == 4 || G == 8 || G == 16 || G == 32, "lanes_per_chain=%d not in {4, 8, 16, 32}", G);
    int V = 1;
    while (G * V < a.d) V *= 2;
    FMC_CHECK_SUPPORTED(V <= 8, "lanes_per_chain=%d too small for n_dim=%d", G, a.d);
    sh = Shape{G, V};
  }
  FMC_CHECK_SUPPORTED(sh.G * sh.V >= a.d, "shape too small for n_dim");
  switch (params->kind) {
    case FMC_KERNEL_MALA: return launch_local_mala(a, sh, st);
    case FMC_KERNEL_HMC: return launch_local_hmc(a, sh, st);
    default: return launch_local_grw(a, sh, st);
  }
}

}  // namespace fmc

using namespace fmc;

extern "C" int fmc_local_steps(const FmcTarget* target, const FmcLocalParams* params, const float* x0,
                               const float* lp0, int32_t n_chains, int32_t n_steps, int32_t thinning, uint64_t seed,
                               uint64_t counter, const float* noise, const float* unif, float* out_pos,
                               float* out_logp, float* out_acc, int64_t buf_len, int64_t cursor,
                               float* x_last, float* lp_last, void* stream) {
  int rc = check_target(target);
  if (rc) return rc;
  FMC_CHECK_ARG(params != nullptr, "params is NULL");
  FMC_CHECK_ARG(params->kind >= 0 && params->kind <= FMC_KERNEL_GRW, "unknown kernel kind %d", params->kind);
  FMC_CHECK_ARG(n_chains >= 0, "n_chains=%d < 0", n_chains);
  FMC_CHECK_ARG(n_steps >= 1, "n_steps=%d < 1", n_steps);
  FMC_CHECK_ARG(thinning >= 1, "thinning=%d < 1", thinning);
  FMC_CHECK_ARG(params->kind != FMC_KERNEL_HMC || params->n_leapfrog >= 0, "n_leapfrog < 0");
  const int64_t n_rec = ((int64_t)n_steps + thinning - 1) / thinning;
  FMC_CHECK_ARG(n_rec <= buf_len, "update of %lld rows does not fit a buffer of %lld rows",
                (long long)n_rec, (long long)buf_len);
  FMC_CHECK_ARG(cursor >= 0, "cursor < 0");
  if (n_chains == 0) return FMC_OK;
  FMC_CHECK_ARG(x0 && out_pos && out_logp && out_acc && x_last && lp_last, "NULL array argument");
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
  a.lp0 = lp0;
  a.C = n_chains;
  a.d = target->n_dim;
  a.S = n_steps;
  a.thin = thinning;
  FMC_CHECK_ARG(params->philox_rounds == 0 || params->philox_rounds == 7 || params->philox_rounds == 10,
                "philox_rounds must be 0, 7 or 10");
  a.rng = Rng{(uint32_t)seed, (uint32_t)(seed >> 32), counter, rng_epoch(), params->philox_rounds == 7 ? 7 : 10};
  a.noise = noise;
  a.unif = unif;
  a.out_pos = out_pos;
  a.out_logp = out_logp;
  a.out_acc = out_acc;
  a.buf_len = buf_len;
  a.start = cursor < buf_len - n_rec ? cursor : buf_len - n_rec;
  a.x_last = x_last;
  a.lp_last = lp_last;

  return dispatch_local(a, params, (cudaStream_t)stream);
}

template <int TGT, int G, int V>
static int launch_eval_t(const FmcTarget& t, const float* x, int64_t n, float* logp, float* grad, cudaStream_t st) {
  const int threads = 256, gpb = threads / G, gpw = 32 / G;
  const int64_t n_pad = (n + gpw - 1) / gpw * gpw;
  const size_t smem = (TGT == FMC_TARGET_DENSE_GAUSSIAN) ? (size_t)gpb * t.n_dim * sizeof(float) : 0;
  int64_t blocks = (n_pad + gpb - 1) / gpb;
  const int64_t cap = (int64_t)sm_count() * 8;
  if (blocks > cap) blocks = cap;
  k_target_eval<TGT, G, V><<<(int)blocks, threads, smem, st>>>(t, x, n, n_pad, logp, grad);
  FMC_LAUNCH_CHECK();
  return FMC_OK;
}

template <int TGT>
static int launch_eval_tgt(const FmcTarget& t, const float* x, int64_t n, float* logp, float* grad, cudaStream_t st) {
  const Shape sh = default_shape(t.n_dim);
#define FMC_EVAL_CASE(g, v) \
  if (sh.G == g && sh.V == v) return launch_eval_t<TGT, g, v>(t, x, n, logp, grad, st);
  FMC_EVAL_CASE(4, 1) FMC_EVAL_CASE(8, 1) FMC_EVAL_CASE(8, 2) FMC_EVAL_CASE(8, 4)
  FMC_EVAL_CASE(16, 4) FMC_EVAL_CASE(32, 4) FMC_EVAL_CASE(32, 8)
#undef FMC_EVAL_CASE
  set_error("no evaluation shape for n_dim=%d", t.n_dim);
  return FMC_ERR_UNSUPPORTED;
}

extern "C" int fmc_target_value_grad(const FmcTarget* target, const float* x, int64_t n, float* logp,
                                     float* grad, void* stream) {
  int rc = check_target(target);
  if (rc) return rc;
  FMC_CHECK_ARG(n >= 0, "n < 0");
  if (n == 0) return FMC_OK;
  FMC_CHECK_ARG(x && logp, "NULL array argument");
  if (target->kind == FMC_TARGET_DENSE_GAUSSIAN)
    FMC_CHECK_SUPPORTED(target->n_dim <= 128, "dense Gaussian group kernel supports n_dim <= 128");
  cudaStream_t st = (cudaStream_t)stream;
  switch (target->kind) {
    case FMC_TARGET_DIAG_GAUSSIAN: return launch_eval_tgt<FMC_TARGET_DIAG_GAUSSIAN>(*target, x, n, logp, grad, st);
    case FMC_TARGET_DUAL_MOON: return launch_eval_tgt<FMC_TARGET_DUAL_MOON>(*target, x, n, logp, grad, st);
    case FMC_TARGET_GAUSS_MIXTURE: return launch_eval_tgt<FMC_TARGET_GAUSS_MIXTURE>(*target, x, n, logp, grad, st);
    case FMC_TARGET_ROSENBROCK: return launch_eval_tgt<FMC_TARGET_ROSENBROCK>(*target, x, n, logp, grad, st);
    default: return launch_eval_tgt<FMC_TARGET_DENSE_GAUSSIAN>(*target, x, n, logp, grad, st);
  }
}
