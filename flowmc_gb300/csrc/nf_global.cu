// nf_global.cu -- K5: the NFProposal global step (resource/kernel/NF_proposal.py:27-172)
// for all chains at once.
//
//   1. flow sample of n_chains * n_steps proposals (rqSpline.py:490-496;
//      base normals from Philox or explicit)
//   2. flow log_prob of the proposals and of the current positions in one
//      pass (NF_proposal.py:44, 165-166: the proposals' flow density is
//      recomputed by the forward pass, not taken from the inverse)
//   3. k_nf_accept: per chain (a lane group, as in the local-step kernel),
//      the target log-density of each proposal, the sequential
//      independent-MH scan (NF_proposal.py:91-126) and the thinned buffer
//      writes, fused in one kernel.
#include "flow.cuh"
#include "targets.cuh"

namespace fmc {

int flow_apply_logprob(const FmcFlow* f, const float* x, int64_t n, float* logp, void* ws, size_t ws_bytes,
                       cudaStream_t st);
int flow_sample_rows(const FmcFlow* f, uint64_t seed, uint64_t counter, const float* z, int64_t n, float* x, void* ws,
                     size_t ws_bytes, cudaStream_t st);
size_t flow_infer_ws_bytes(const FmcFlow* f, int64_t n);

struct NfArgs {
  FmcTarget tgt;
  const float* x0;      // [C, d]
  const float* props;   // [C*S, d]
  const float* lnf;     // [C*S + C]: proposals then current positions
  int32_t C, d, S, thin;
  Rng rng;
  const float* unif;
  float *out_pos, *out_logp, *out_acc;
  int64_t buf_len, start;
  float *x_last, *lp_last;
  int64_t C_pad;
};

template <int TGT, int G, int V>
__global__ void __launch_bounds__(256) k_nf_accept(const NfArgs a) {
  extern __shared__ float smem[];
  const int gl = threadIdx.x % G;
  const int64_t gpb = blockDim.x / G, gib = threadIdx.x / G;
  const int d = a.d;
  float* stage = (TGT == FMC_TARGET_DENSE_GAUSSIAN) ? smem + gib * d : nullptr;
  const Rng rng = a.rng.at_epoch();
  for (int64_t c = blockIdx.x * gpb + gib; c < a.C_pad; c += (int64_t)gridDim.x * gpb) {
    const bool active = c < a.C;
    const int64_t cc = active ? c : 0;
    float x[V], g[V];
#pragma unroll
    for (int v = 0; v < V; ++v) {
      const int j = gl * V + v;
      x[v] = (j < d) ? __ldg(a.x0 + cc * d + j) : 0.f;
    }
    float lp = target_eval<TGT, G, V, false>(a.tgt, x, g, gl, stage);   // take_steps.py:201-203
    float lnf = __ldg(a.lnf + (int64_t)a.C * a.S + cc);
    float xr[V], lpr = lp;
#pragma unroll
    for (int v = 0; v < V; ++v) xr[v] = x[v];
    for (int s = 0; s < a.S; ++s) {
      const int64_t row = cc * a.S + s;
      float p[V];
#pragma unroll
      for (int v = 0; v < V; ++v) {
        const int j = gl * V + v;
        p[v] = (j < d) ? __ldg(a.props + row * d + j) : 0.f;
      }
      const float lpp = target_eval<TGT, G, V, false>(a.tgt, p, g, gl, stage);
      const float lnfp = __ldg(a.lnf + row);
      const float u = a.unif ? __ldg(a.unif + row) : u32_to_unit(rng.draw(cc, s, 0u, RNG_TAG_NF_UNIFORM).x);
      // ratio = (lp_p - lp_c) - (lnf_p - lnf_c)   (NF_proposal.py:102-104)
      const ff ratio = ff_add(two_sum(lpp, -lp), ff_neg(two_sum(lnfp, -lnf)));
      const bool acc = f_lt_ff(logf(u), ratio);
      if (acc) {
#pragma unroll
        for (int v = 0; v < V; ++v) x[v] = p[v];
        lp = lpp;
        lnf = lnfp;
      }
      if (s % a.thin == 0) {
        if (active) {
          const int64_t orow = cc * a.buf_len + a.start + s / a.thin;
#pragma unroll
          for (int v = 0; v < V; ++v) {
            const int j = gl * V + v;
            if (j < d) __stcs(a.out_pos + orow * d + j, x[v]);
          }
          if (gl == 0) {
            __stcs(a.out_logp + orow, lp);
            __stcs(a.out_acc + orow, acc ? 1.f : 0.f);
          }
        }
#pragma unroll
        for (int v = 0; v < V; ++v) xr[v] = x[v];
        lpr = lp;
      }
    }
    if (active) {
#pragma unroll
      for (int v = 0; v < V; ++v) {
        const int j = gl * V + v;
        if (j < d) a.x_last[cc * d + j] = xr[v];
      }
      if (gl == 0 && a.lp_last) a.lp_last[cc] = lpr;
    }
  }
}

template <int TGT, int G, int V>
static int launch_nf_t(const NfArgs& a0, cudaStream_t st) {
  NfArgs a = a0;
  const int threads = 256, gpb = threads / G, gpw = 32 / G;
  a.C_pad = ((int64_t)a.C + gpw - 1) / gpw * gpw;
  const size_t smem = (TGT == FMC_TARGET_DENSE_GAUSSIAN) ? (size_t)gpb * a.d * sizeof(float) : 0;
  int64_t blocks = (a.C_pad + gpb - 1) / gpb;
  const int64_t cap = (int64_t)sm_count() * 8;
  if (blocks > cap) blocks = cap;
  // proposals and their flow densities read, thinned rows written
  const double n_rec = (double)((a.S + a.thin - 1) / a.thin);
  KernelTimer kt(FMC_KT_NF_ACCEPT, st, 0.0,
                 (double)a.C * a.S * (4.0 * a.d + 4.0) + (double)a.C * n_rec * (4.0 * a.d + 8.0));
  k_nf_accept<TGT, G, V><<<(int)blocks, threads, smem, st>>>(a);
  FMC_LAUNCH_CHECK();
  return FMC_OK;
}

template <int TGT>
static int launch_nf_tgt(const NfArgs& a, cudaStream_t st) {
  const int d = a.d;
#define NFC(g, v, lim) \
  if (d <= lim) return launch_nf_t<TGT, g, v>(a, st);
  NFC(4, 1, 4) NFC(8, 1, 8) NFC(8, 2, 16) NFC(8, 4, 32) NFC(16, 4, 64) NFC(32, 4, 128) NFC(32, 8, 256)
#undef NFC
  set_error("n_dim=%d too large for the global-step kernel", d);
  return FMC_ERR_UNSUPPORTED;
}

int check_target(const FmcTarget* t);

static size_t a256(size_t v) { return (v + 255) / 256 * 256; }

}  // namespace fmc

using namespace fmc;

extern "C" int fmc_nf_workspace_size(const FmcFlow* flow, int32_t n_chains, int32_t n_steps, size_t* bytes) {
  FMC_CHECK_ARG(flow && bytes, "NULL pointer");
  FMC_CHECK_ARG(n_chains >= 1 && n_steps >= 1, "bad sizes");
  const int64_t rows = (int64_t)n_chains * n_steps;
  const int d = flow->n_dim;
  *bytes = a256((size_t)(rows + n_chains) * d * 4) + a256((size_t)(rows + n_chains) * 4) +
           flow_infer_ws_bytes(flow, rows + n_chains);
  return FMC_OK;
}

// the accept scan over precomputed proposals props [C * S, d] (row c * S + s)
// and flow log-densities lnf [C * S + C] (the proposals', then the current
// positions')
static int launch_accept(const FmcTarget* target, const float* x0, int32_t n_chains, int32_t n_steps,
                         int32_t thinning, uint64_t seed, uint64_t counter, const float* props, const float* lnf,
                         const float* unif, float* out_pos, float* out_logp, float* out_acc, int64_t buf_len,
                         int64_t cursor, float* x_last, float* lp_last, cudaStream_t st) {
  const int64_t n_rec = ((int64_t)n_steps + thinning - 1) / thinning;
  NfArgs a{};
  a.tgt = *target;
  a.x0 = x0;
  a.props = props;
  a.lnf = lnf;
  a.C = n_chains;
  a.d = target->n_dim;
  a.S = n_steps;
  a.thin = thinning;
  a.rng = Rng{(uint32_t)seed, (uint32_t)(seed >> 32), counter, rng_epoch()};
  a.unif = unif;
  a.out_pos = out_pos;
  a.out_logp = out_logp;
  a.out_acc = out_acc;
  a.buf_len = buf_len;
  a.start = cursor < buf_len - n_rec ? cursor : buf_len - n_rec;
  a.x_last = x_last;
  a.lp_last = lp_last;
  switch (target->kind) {
    case FMC_TARGET_DIAG_GAUSSIAN: return launch_nf_tgt<FMC_TARGET_DIAG_GAUSSIAN>(a, st);
    case FMC_TARGET_DUAL_MOON: return launch_nf_tgt<FMC_TARGET_DUAL_MOON>(a, st);
    case FMC_TARGET_GAUSS_MIXTURE: return launch_nf_tgt<FMC_TARGET_GAUSS_MIXTURE>(a, st);
    case FMC_TARGET_ROSENBROCK: return launch_nf_tgt<FMC_TARGET_ROSENBROCK>(a, st);
    default: return launch_nf_tgt<FMC_TARGET_DENSE_GAUSSIAN>(a, st);
  }
}

extern "C" int fmc_nf_global_steps(const FmcFlow* flow, const FmcTarget* target, const float* x0, int32_t n_chains,
                                   int32_t n_steps, int32_t thinning, uint64_t seed, uint64_t counter,
                                   const float* z, const float* unif, float* out_pos, float* out_logp,
                                   float* out_acc, int64_t buf_len, int64_t cursor, float* x_last, float* lp_last,
                                   void* ws, size_t ws_bytes, void* stream) {
  int rc = check_target(target);
  if (rc) return rc;
  FMC_CHECK_ARG(flow != nullptr, "flow is NULL");
  FMC_CHECK_ARG(flow->n_dim == target->n_dim, "flow n_dim %d != target n_dim %d", flow->n_dim, target->n_dim);
  FMC_CHECK_ARG(n_chains >= 0 && n_steps >= 1 && thinning >= 1, "bad sizes");
  const int64_t n_rec = ((int64_t)n_steps + thinning - 1) / thinning;
  FMC_CHECK_ARG(n_rec <= buf_len, "update of %lld rows does not fit a buffer of %lld rows", (long long)n_rec,
                (long long)buf_len);
  FMC_CHECK_ARG(cursor >= 0, "cursor < 0");
  if (n_chains == 0) return FMC_OK;
  FMC_CHECK_ARG(x0 && out_pos && out_logp && out_acc && x_last, "NULL array argument");
  size_t need = 0;
  if ((rc = fmc_nf_workspace_size(flow, n_chains, n_steps, &need))) return rc;
  FMC_CHECK_ARG(ws && ws_bytes >= need, "workspace of %zu bytes < %zu needed", ws_bytes, need);
  FMC_CHECK_ARG(((uintptr_t)ws & 255) == 0, "workspace must be 256-byte aligned");
  if (target->kind == FMC_TARGET_DENSE_GAUSSIAN)
    FMC_CHECK_SUPPORTED(target->n_dim <= 128, "dense Gaussian group kernel supports n_dim <= 128");
  cudaStream_t st = (cudaStream_t)stream;
  const int d = flow->n_dim;
  const int64_t rows = (int64_t)n_chains * n_steps;
  char* p = (char*)ws;
  float* props = (float*)p;  // [rows + C, d]: proposals, then the current positions
  p += a256((size_t)(rows + n_chains) * d * 4);
  float* lnf = (float*)p;
  p += a256((size_t)(rows + n_chains) * 4);
  void* fws = p;
  const size_t fws_bytes = ws_bytes - (size_t)(p - (char*)ws);

  if ((rc = flow_sample_rows(flow, seed, counter, z, rows, props, fws, fws_bytes, st))) return rc;
  FMC_CUDA_TRY(cudaMemcpyAsync(props + rows * d, x0, (size_t)n_chains * d * 4, cudaMemcpyDeviceToDevice, st));
  if ((rc = flow_apply_logprob(flow, props, rows + n_chains, lnf, fws, fws_bytes, st))) return rc;

  return launch_accept(target, x0, n_chains, n_steps, thinning, seed, counter, props, lnf, unif, out_pos, out_logp,
                       out_acc, buf_len, cursor, x_last, lp_last, st);
}

extern "C" int fmc_nf_accept(const FmcTarget* target, const float* x0, int32_t n_chains, int32_t n_steps,
                             int32_t thinning, uint64_t seed, uint64_t counter, const float* props, const float* lnf,
                             const float* unif, float* out_pos, float* out_logp, float* out_acc, int64_t buf_len,
                             int64_t cursor, float* x_last, float* lp_last, void* stream) {
  int rc = check_target(target);
  if (rc) return rc;
  FMC_CHECK_ARG(n_chains >= 0 && n_steps >= 1 && thinning >= 1, "bad sizes");
  const int64_t n_rec = ((int64_t)n_steps + thinning - 1) / thinning;
  FMC_CHECK_ARG(n_rec <= buf_len, "update of %lld rows does not fit a buffer of %lld rows", (long long)n_rec,
                (long long)buf_len);
  FMC_CHECK_ARG(cursor >= 0, "cursor < 0");
  if (n_chains == 0) return FMC_OK;
  FMC_CHECK_ARG(x0 && props && lnf && out_pos && out_logp && out_acc && x_last, "NULL array argument");
  if (target->kind == FMC_TARGET_DENSE_GAUSSIAN)
    FMC_CHECK_SUPPORTED(target->n_dim <= 128, "dense Gaussian group kernel supports n_dim <= 128");
  return launch_accept(target, x0, n_chains, n_steps, thinning, seed, counter, props, lnf, unif, out_pos, out_logp,
                       out_acc, buf_len, cursor, x_last, lp_last, (cudaStream_t)stream);
}
