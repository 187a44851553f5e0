// local_steps.cuh -- K1: the persistent local-step kernel.
//
// One launch runs n_steps of MALA, HMC or Gaussian random walk for every
// chain. A chain is owned by a group of G lanes (lanes_per_chain) that keep
// its position, log-density and gradient in registers for the whole call;
// noise comes from in-kernel Philox (or an explicit array for parity runs),
// the Metropolis-Hastings accept is fused in, and every `thinning`-th state
// is written straight into flowMC's buffers [n_chains, buf_len, n_dim] with
// vectorised streaming stores (the G lanes of a chain cover one contiguous
// row, so the store of a step is one coalesced segment).
//
// Reference semantics reproduced (flowMC v0.4.5):
//  * TakeSerialSteps.sample: lp0 = logpdf(x0); scan over steps
//    (strategy/take_steps.py:164-180); thinning positions[:, ::thinning]
//    (take_steps.py:134-138); the strategy returns the last *thinned*
//    position (take_steps.py:144).
//  * MALA.kernel (resource/kernel/MALA.py:26-89): proposal
//    x + dt^2 g(x)/2 + dt xi, log-ratio with the two isotropic Gaussian
//    proposal densities, accept iff log(u) < ratio, lp recomputed at x.
//    The (lp0, g0) the reference recomputes every step equals the cached
//    value of the previous step bit for bit, so it is cached here.
//  * HMC.kernel (resource/kernel/HMC.py:98-151): momentum xi @
//    cholesky(inv(M)).T, kinetic 0.5 * sum(p^2 * M) (broadcast: column sums
//    of M), leapfrog table rows [0,.5], [1,1] x n_leapfrog, [1,.5]
//    (HMC.py:47-50, 71-80) = n_leapfrog+1 drifts with half kicks at both
//    ends; H uses the incoming log_prob (HMC.py:137).
//  * GaussianRandomWalk.kernel (Gaussian_random_walk.py:48-61).
//
// The MH log-ratio is assembled in float-float arithmetic (about 48
// significant bits) instead of FP64: this GPU's FP64 rate is too low for a
// per-chain-step operation, and the inputs (lp, squared norms) are FP32.
#pragma once
#include "targets.cuh"

namespace fmc {

struct LocalArgs {
  FmcTarget tgt;
  int32_t n_leapfrog;
  float step;
  const float* mscale;  // HMC momentum scale (diag of cholesky(inv(M)))
  const float* mcol;    // HMC column sums of M
  const float* mchol;   // HMC with a dense M: cholesky(inv(M)) [d, d] row-major, or NULL
  int32_t mstage_off;   // floats of dynamic shared memory before the momentum staging
  const float* x0;
  const float* lp0;
  int32_t C, d, S, thin;
  Rng rng;
  const float* noise;
  const float* unif;
  float* out_pos;
  float* out_logp;
  float* out_acc;
  int64_t buf_len, start;
  float* x_last;
  float* lp_last;
  int64_t C_pad;
  int32_t tab_smem;   // diag Gaussian / mixture: tables staged in shared memory
  // parallel tempering (NULL temps: plain target). Row c targets
  // beta * log L(x) + log prior(x) with beta = 1 / temps[c % n_temps]; the
  // prior is zero or diagonal Gaussian (prior_iv != NULL).
  const float* temps;
  int32_t n_temps;
  const float* prior_mean;
  const float* prior_iv;
  float prior_const;
  float* acc_count;   // optional: accepted steps per chain
};

// Tempered log-density (resource/logPDF.py:106-108): (1 / T) * log L(x) +
// log prior(x), with the gradient scaled the same way.
template <int G, int V, bool GRAD>
__device__ __forceinline__ float temper(const LocalArgs& a, float lp, const float (&x)[V], float (&g)[V],
                                        float beta, int gl) {
  lp = beta * lp;
  if constexpr (GRAD) {
#pragma unroll
    for (int v = 0; v < V; ++v) g[v] *= beta;
  }
  if (a.prior_iv) {
    float s = 0.f;
#pragma unroll
    for (int v = 0; v < V; ++v) {
      const int j = gl * V + v;
      if (j < a.d) {
        const float dx = x[v] - __ldg(a.prior_mean + j);
        const float iv = __ldg(a.prior_iv + j);
        s += dx * dx * iv;
        if constexpr (GRAD) g[v] -= dx * iv;
      }
    }
    lp += -0.5f * group_sum<G>(s) + a.prior_const;
  }
  return lp;
}

template <int V>
__device__ __forceinline__ void draw_normals(const LocalArgs& a, const Rng& rng, int64_t c, int s, int gl,
                                             float (&xi)[V]) {
  const int d = a.d;
  if (a.noise) {
    const float* row = a.noise + ((int64_t)c * a.S + s) * d;
#pragma unroll
    for (int v = 0; v < V; ++v) {
      const int j = gl * V + v;
      xi[v] = (j < d) ? __ldcs(row + j) : 0.f;
    }
    return;
  }
  // Coordinate j takes component (j & 3) of the Philox block keyed by j & ~3:
  // (x, y) -> Box-Muller -> j&3 = 0, 1 and (z, w) -> j&3 = 2, 3. The stream
  // depends on (chain, step, coordinate) only, never on the lane-group shape,
  // so every (G, V) choice samples the same chains.
  if constexpr (V >= 4) {
#pragma unroll
    for (int q = 0; q < V; q += 4) {
      const u32x4 r = rng.draw(c, s, (uint32_t)(gl * V + q), RNG_TAG_LOCAL_NORMAL);
      box_muller(r.x, r.y, xi[q], xi[q + 1]);
      box_muller(r.z, r.w, xi[q + 2], xi[q + 3]);
    }
  } else {
    const int j = gl * V;   // V = 2: j is even
    const u32x4 r = rng.draw(c, s, (uint32_t)(j & ~3), RNG_TAG_LOCAL_NORMAL);
    const bool hi = (j & 2) != 0;
    float z0, z1;
    box_muller(hi ? r.z : r.x, hi ? r.w : r.y, z0, z1);
    if constexpr (V == 1) {
      xi[0] = (j & 1) ? z1 : z0;
    } else {
      xi[0] = z0;
      xi[1] = z1;
    }
  }
#pragma unroll
  for (int v = 0; v < V; ++v)
    if (gl * V + v >= d) xi[v] = 0.f;
}

// Uniforms: step s takes component s & 3 of the Philox block keyed by s >> 2.
// The G lanes of a group share the work: on steps s = 0 mod 4G, lane gl
// computes block (s >> 2) + gl into `ub`, and each step the owner lane
// ((s >> 2) mod G) hands its component to the whole group with a shuffle,
// so the group agrees on u. One Philox call per 4G steps per lane instead of
// one per 4 steps; the stream is the same as one lane drawing every block.
template <int G>
__device__ __forceinline__ float draw_uniform(const LocalArgs& a, const Rng& rng, int64_t c, int s, int gl,
                                              u32x4& ub) {
  if (a.unif) return __ldcs(a.unif + (int64_t)c * a.S + s);
  if (s % (4 * G) == 0) ub = rng.draw(c, (uint64_t)((s >> 2) + gl), 0u, RNG_TAG_LOCAL_UNIFORM);
  const int r = s & 3;
  const uint32_t mine = r == 0 ? ub.x : r == 1 ? ub.y : r == 2 ? ub.z : ub.w;
  return u32_to_unit(__shfl_sync(0xffffffffu, mine, (s >> 2) % G, G));
}

template <int G, int V>
__device__ __forceinline__ void store_row(float* dst, const float (&x)[V], int gl, int d) {
  // dst points at element 0 of the row. With d a multiple of the vector
  // width, each vector chunk of a lane's coordinates is wholly inside the row
  // or wholly padding, so the guard is per chunk (a lane may straddle d).
  if constexpr (V % 4 == 0) {
    if (d % 4 == 0) {
#pragma unroll
      for (int q = 0; q < V; q += 4)
        if (gl * V + q < d)
          __stcs(reinterpret_cast<float4*>(dst + gl * V + q), make_float4(x[q], x[q + 1], x[q + 2], x[q + 3]));
      return;
    }
  }
  if constexpr (V % 2 == 0) {
    if (d % 2 == 0) {
#pragma unroll
      for (int q = 0; q < V; q += 2)
        if (gl * V + q < d) __stcs(reinterpret_cast<float2*>(dst + gl * V + q), make_float2(x[q], x[q + 1]));
      return;
    }
  }
#pragma unroll
  for (int v = 0; v < V; ++v) {
    const int j = gl * V + v;
    if (j < d) __stcs(dst + j, x[v]);
  }
}

// Resident blocks per SM the kernel's registers must leave room for (0: no
// bound given). Three for MALA with 8 coordinates per lane on the Rosenbrock
// and mixture targets: at most 80 registers a thread, bit-identical results,
// measured 10 % / 3 % faster on GB300 than two blocks at 114-127 registers.
// HMC and the other targets spill under the same cap and keep the default.
template <int KIND, int TGT, int V>
constexpr int local_min_blocks() {
  return (KIND == FMC_KERNEL_MALA && V >= 8 && (TGT == FMC_TARGET_ROSENBROCK || TGT == FMC_TARGET_GAUSS_MIXTURE))
             ? 3
             : 0;
}

template <int KIND, int TGT, int G, int V>
__global__ void __launch_bounds__(256, local_min_blocks<KIND, TGT, V>()) k_local_steps(const LocalArgs a) {
  extern __shared__ float smem[];
  const int gl = threadIdx.x % G;
  const int64_t groups_per_block = blockDim.x / G;
  const int64_t gib = threadIdx.x / G;
  const int d = a.d;
  float* stage = (TGT == FMC_TARGET_DENSE_GAUSSIAN) ? smem + gib * d : nullptr;
  if constexpr (TGT == FMC_TARGET_DIAG_GAUSSIAN || TGT == FMC_TARGET_GAUSS_MIXTURE) {
    if (a.tab_smem) {
      stage_target_table(a.tgt, smem);
      __syncthreads();
      stage = smem;
    }
  }
  const float dt = a.step;
  const Rng rng = a.rng.at_epoch();

  for (int64_t c = blockIdx.x * groups_per_block + gib; c < a.C_pad;
       c += (int64_t)gridDim.x * groups_per_block) {
    const bool active = c < a.C;
    const int64_t cc = active ? c : 0;
    float x[V], g[V];
#pragma unroll
    for (int v = 0; v < V; ++v) {
      const int j = gl * V + v;
      x[v] = (j < d) ? __ldg(a.x0 + cc * d + j) : 0.f;
    }
    const bool tempered = a.temps != nullptr;
    const float beta = tempered ? __fdiv_rn(1.f, __ldg(a.temps + cc % a.n_temps)) : 1.f;
    float lp = target_eval<TGT, G, V, KIND != FMC_KERNEL_GRW>(a.tgt, x, g, gl, stage);
    if (tempered) lp = temper<G, V, KIND != FMC_KERNEL_GRW>(a, lp, x, g, beta, gl);
    if (KIND != FMC_KERNEL_MALA && a.lp0 != nullptr) lp = __ldg(a.lp0 + cc);
    float xr[V], lpr = lp;
#pragma unroll
    for (int v = 0; v < V; ++v) xr[v] = x[v];

    u32x4 ub{0u, 0u, 0u, 0u};
    // next stored row (every thin-th step, from row `start`); no rows are
    // stored when out_pos is NULL (the tempered chains keep only their end)
    const bool rec = a.out_pos != nullptr;
    const int64_t row0 = cc * a.buf_len + a.start;
    float* prow = rec ? a.out_pos + row0 * d : nullptr;
    float* plp = rec ? a.out_logp + row0 : nullptr;
    float* pacc = rec ? a.out_acc + row0 : nullptr;
    int tcount = 0, n_acc = 0;
    for (int s = 0; s < a.S; ++s) {
      float xi[V];
      draw_normals<V>(a, rng, cc, s, gl, xi);
      const float logu = logf(draw_uniform<G>(a, rng, cc, s, gl, ub));
      bool acc;
      if constexpr (KIND == FMC_KERNEL_MALA) {
        const float dt2 = dt * dt;
        float mean0[V], prop[V], g1[V];
#pragma unroll
        for (int v = 0; v < V; ++v) {
          mean0[v] = x[v] + dt2 * g[v] / 2.0f;
          prop[v] = mean0[v] + dt * xi[v];
        }
        float lp1 = target_eval<TGT, G, V, true>(a.tgt, prop, g1, gl, stage);
        if (tempered) lp1 = temper<G, V, true>(a, lp1, prop, g1, beta, gl);
        float sa = 0.f, sb = 0.f;
#pragma unroll
        for (int v = 0; v < V; ++v) {
          const float ea = prop[v] - mean0[v];
          const float eb = x[v] - (prop[v] + dt2 * g1[v] / 2.0f);
          sa += ea * ea;
          sb += eb * eb;
        }
        sa = group_sum<G>(sa);
        sb = group_sum<G>(sb);
        // ratio = (lp1 - lp0) - log q(prop | x) + log q(x | prop)
        //       = (lp1 - lp0) + (|prop - mean0|^2 - |x - mean1|^2) / (2 dt^2)
        // (the Gaussian normalisers cancel). Decided in float32 when log u
        // is farther from the float32 ratio than that ratio's rounding error
        // can reach; otherwise in float-float (accepts identical either way).
        const float c2 = 0.5f / dt2;
        const float rf = (lp1 - lp) + (sa - sb) * c2;
        const float bound = 4.8e-7f * (fabsf(lp1) + fabsf(lp) + (sa + sb) * c2) + 1e-30f;
        if (fabsf(logu - rf) > bound) {
          acc = logu < rf;
        } else {
          const ff q = two_sum(sa, -sb);
          const ff ratio = ff_add(two_sum(lp1, -lp), ff_mul_f(q, c2));
          acc = f_lt_ff(logu, ratio);
        }
        if (acc) {
#pragma unroll
          for (int v = 0; v < V; ++v) { x[v] = prop[v]; g[v] = g1[v]; }
          lp = lp1;
        }
      } else if constexpr (KIND == FMC_KERNEL_HMC) {
        float p[V], mc[V], xq[V], gq[V];
        float k0 = 0.f;
        if (a.mchol) {
          // dense metric: p = xi @ L^T (HMC.py:133-136), the chain's normals
          // shared through this group's slice of shared memory
          float* xs = smem + a.mstage_off + gib * d;
#pragma unroll
          for (int v = 0; v < V; ++v)
            if (gl * V + v < d) xs[gl * V + v] = xi[v];
          __syncwarp();
#pragma unroll
          for (int v = 0; v < V; ++v) {
            const int j = gl * V + v;
            float acc = 0.f;
            if (j < d) {
              const float* Lr = a.mchol + (int64_t)j * d;
              for (int k = 0; k <= j; ++k) acc = fmaf(__ldg(Lr + k), xs[k], acc);   // L is lower triangular
            }
            p[v] = acc;
          }
          __syncwarp();   // xs is rewritten at the next step
        } else {
#pragma unroll
          for (int v = 0; v < V; ++v) {
            const int j = gl * V + v;
            p[v] = xi[v] * ((j < d) ? ldg_or(a.mscale, j, 1.f) : 0.f);
          }
        }
#pragma unroll
        for (int v = 0; v < V; ++v) {
          const int j = gl * V + v;
          const bool in = j < d;
          mc[v] = in ? ldg_or(a.mcol, j, 1.f) : 0.f;
          k0 += p[v] * p[v] * mc[v];
          xq[v] = x[v];
        }
        k0 = 0.5f * group_sum<G>(k0);
        // row 0: drift coefficient 0, kick 0.5 with the gradient at x
        const float e0 = dt * 0.5f;
#pragma unroll
        for (int v = 0; v < V; ++v) p[v] = p[v] + e0 * g[v];
        // rows 1..n_leapfrog: drift and full kick; only the gradient is used,
        // so the log-density (and its group reduction) is left to the
        // compiler to drop
        const int nlf = a.n_leapfrog;
        for (int r = 1; r <= nlf; ++r) {
#pragma unroll
          for (int v = 0; v < V; ++v) xq[v] = xq[v] + dt * (p[v] * mc[v]);
          float lpi = target_eval<TGT, G, V, true>(a.tgt, xq, gq, gl, stage);
          if (tempered) lpi = temper<G, V, true>(a, lpi, xq, gq, beta, gl);
          (void)lpi;
#pragma unroll
          for (int v = 0; v < V; ++v) p[v] = p[v] + dt * gq[v];
        }
        // last row: drift, half kick, and the log-density at the end point
#pragma unroll
        for (int v = 0; v < V; ++v) xq[v] = xq[v] + dt * (p[v] * mc[v]);
        float lpq = target_eval<TGT, G, V, true>(a.tgt, xq, gq, gl, stage);
        if (tempered) lpq = temper<G, V, true>(a, lpq, xq, gq, beta, gl);
        {
          const float eh = dt * 0.5f;
#pragma unroll
          for (int v = 0; v < V; ++v) p[v] = p[v] + eh * gq[v];
        }
        float k1 = 0.f;
#pragma unroll
        for (int v = 0; v < V; ++v) k1 += p[v] * p[v] * mc[v];
        k1 = 0.5f * group_sum<G>(k1);
        // log_acc = (-lp + K0) - (-lpq + K1), decided in float32 away from
        // the float32 rounding band, else in float-float (as for MALA)
        const float rf = (lpq - lp) + (k0 - k1);
        const float bound = 4.8e-7f * (fabsf(lp) + fabsf(lpq) + k0 + k1) + 1e-30f;
        if (fabsf(logu - rf) > bound) {
          acc = logu < rf;
        } else {
          const ff h0 = two_sum(-lp, k0);
          const ff h1 = two_sum(-lpq, k1);
          const ff log_acc = ff_add(h0, ff_neg(h1));
          acc = f_lt_ff(logu, log_acc);
        }
        if (acc) {
#pragma unroll
          for (int v = 0; v < V; ++v) { x[v] = xq[v]; g[v] = gq[v]; }
          lp = lpq;
        }
      } else {  // GRW
        float prop[V], gdummy[V];
#pragma unroll
        for (int v = 0; v < V; ++v) prop[v] = x[v] + xi[v] * dt;
        float lpp = target_eval<TGT, G, V, false>(a.tgt, prop, gdummy, gl, stage);
        if (tempered) lpp = temper<G, V, false>(a, lpp, prop, gdummy, beta, gl);
        acc = f_lt_ff(logu, two_sum(lpp, -lp));
        if (acc) {
#pragma unroll
          for (int v = 0; v < V; ++v) x[v] = prop[v];
          lp = lpp;
        }
      }
      n_acc += acc ? 1 : 0;
      if (tcount == 0) {
        if (rec) {
          if (active) {
            store_row<G, V>(prow, x, gl, d);
            if (gl == 0) {
              __stcs(plp, lp);
              __stcs(pacc, acc ? 1.f : 0.f);
            }
          }
          prow += d;
          ++plp;
          ++pacc;
        }
#pragma unroll
        for (int v = 0; v < V; ++v) xr[v] = x[v];
        lpr = lp;
      }
      if (++tcount == a.thin) tcount = 0;
    }
    if (active) {
#pragma unroll
      for (int v = 0; v < V; ++v) {
        const int j = gl * V + v;
        if (j < d) a.x_last[cc * d + j] = xr[v];
      }
      if (gl == 0) {
        a.lp_last[cc] = lpr;
        if (a.acc_count) a.acc_count[cc] = (float)n_acc;
      }
    }
  }
}

// ------------------------------------------------------------------ batch eval
template <int TGT, int G, int V>
__global__ void __launch_bounds__(256) k_target_eval(const FmcTarget t, const float* __restrict__ x,
                                                     int64_t n, int64_t n_pad, float* logp, float* grad) {
  extern __shared__ float smem[];
  const int gl = threadIdx.x % G;
  const int64_t gpb = blockDim.x / G, gib = threadIdx.x / G;
  const int d = t.n_dim;
  float* stage = (TGT == FMC_TARGET_DENSE_GAUSSIAN) ? smem + gib * d : nullptr;
  for (int64_t r = blockIdx.x * gpb + gib; r < n_pad; r += (int64_t)gridDim.x * gpb) {
    const bool active = r < n;
    const int64_t rr = active ? r : 0;
    float xv[V], gv[V];
#pragma unroll
    for (int v = 0; v < V; ++v) {
      const int j = gl * V + v;
      xv[v] = (j < d) ? x[rr * d + j] : 0.f;
    }
    const float lp = target_eval<TGT, G, V, true>(t, xv, gv, gl, stage);
    if (active) {
      if (gl == 0) logp[rr] = lp;
      if (grad) {
#pragma unroll
        for (int v = 0; v < V; ++v) {
          const int j = gl * V + v;
          if (j < d) grad[rr * d + j] = gv[v];
        }
      }
    }
  }
}

// ------------------------------------------------------------------ dispatch
// Instantiated (lanes per chain, coordinates per lane) shapes.
struct Shape { int G, V; };

// choose the default (G, V) for a dimension: the fewest lanes whose capacity
// covers n_dim with at most 8 coordinates per lane, preferring wide groups
// only when the dimension needs them.
inline Shape default_shape(int d) {
  if (d <= 4) return {4, 1};
  if (d <= 8) return {8, 1};
  if (d <= 16) return {8, 2};
  if (d <= 32) return {8, 4};
  if (d <= 64) return {16, 4};
  if (d <= 128) return {32, 4};
  return {32, 8};
}

template <int KIND, int TGT, int G, int V>
int launch_local_t(const LocalArgs& a0, cudaStream_t st) {
  LocalArgs a = a0;
  const int threads = 256;
  const int gpb = threads / G;
  const int gpw = 32 / G;
  a.C_pad = ((int64_t)a.C + gpw - 1) / gpw * gpw;
  size_t smem = (TGT == FMC_TARGET_DENSE_GAUSSIAN) ? (size_t)gpb * a.d * sizeof(float) : 0;
  a.tab_smem = 0;
  if (TGT == FMC_TARGET_DIAG_GAUSSIAN || TGT == FMC_TARGET_GAUSS_MIXTURE) {
    const int K = (TGT == FMC_TARGET_GAUSS_MIXTURE) ? a.tgt.n_comp : 1;
    const size_t tab = (size_t)2 * K * a.d * sizeof(float);
    if (tab <= 32 * 1024) {   // small tables only: keeps several blocks per SM
      smem = tab;
      a.tab_smem = 1;
    }
  }
  a.mstage_off = (int32_t)(smem / sizeof(float));
  if (KIND == FMC_KERNEL_HMC && a.mchol != nullptr) smem += (size_t)gpb * a.d * sizeof(float);
  auto kern = k_local_steps<KIND, TGT, G, V>;
  if (smem > 48 * 1024) {
    FMC_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  }
  int per_sm = 0;
  FMC_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem));
  if (per_sm < 1) per_sm = 1;
  const int64_t need = (a.C_pad + gpb - 1) / gpb;
  const int64_t cap = (int64_t)sm_count() * per_sm;
  const int blocks = (int)(need < cap ? need : cap);
  // algorithmic bytes: the stored rows (float32 position + log-density +
  // acceptance per thinned step), plus the starting state read once
  const double rows = a.out_pos ? (double)a.C * ((a.S + a.thin - 1) / a.thin) : 0.0;
  KernelTimer kt(FMC_KT_LOCAL_STEPS, st, 0.0, rows * (4.0 * a.d + 8.0) + (double)a.C * (4.0 * a.d + 4.0));
  kern<<<blocks, threads, smem, st>>>(a);
  FMC_LAUNCH_CHECK();
  return FMC_OK;
}

template <int KIND, int TGT>
int launch_local_shape(const LocalArgs& a, Shape sh, cudaStream_t st) {
#define FMC_SHAPE_CASE(g, v) \
  if (sh.G == g && sh.V == v) return launch_local_t<KIND, TGT, g, v>(a, st);
  FMC_SHAPE_CASE(4, 1) FMC_SHAPE_CASE(4, 2) FMC_SHAPE_CASE(4, 4) FMC_SHAPE_CASE(4, 8)
  FMC_SHAPE_CASE(8, 1) FMC_SHAPE_CASE(8, 2) FMC_SHAPE_CASE(8, 4) FMC_SHAPE_CASE(8, 8)
  FMC_SHAPE_CASE(16, 1) FMC_SHAPE_CASE(16, 2) FMC_SHAPE_CASE(16, 4) FMC_SHAPE_CASE(16, 8)
  FMC_SHAPE_CASE(32, 1) FMC_SHAPE_CASE(32, 2) FMC_SHAPE_CASE(32, 4) FMC_SHAPE_CASE(32, 8)
#undef FMC_SHAPE_CASE
  set_error("lanes_per_chain=%d with %d coordinates per lane is not instantiated", sh.G, sh.V);
  return FMC_ERR_UNSUPPORTED;
}

template <int KIND>
int launch_local_kind(const LocalArgs& a, Shape sh, cudaStream_t st) {
  switch (a.tgt.kind) {
    case FMC_TARGET_DIAG_GAUSSIAN: return launch_local_shape<KIND, FMC_TARGET_DIAG_GAUSSIAN>(a, sh, st);
    case FMC_TARGET_DUAL_MOON: return launch_local_shape<KIND, FMC_TARGET_DUAL_MOON>(a, sh, st);
    case FMC_TARGET_GAUSS_MIXTURE: return launch_local_shape<KIND, FMC_TARGET_GAUSS_MIXTURE>(a, sh, st);
    case FMC_TARGET_ROSENBROCK: return launch_local_shape<KIND, FMC_TARGET_ROSENBROCK>(a, sh, st);
    case FMC_TARGET_DENSE_GAUSSIAN: return launch_local_shape<KIND, FMC_TARGET_DENSE_GAUSSIAN>(a, sh, st);
  }
  set_error("unknown target kind %d", a.tgt.kind);
  return FMC_ERR_INVALID_ARG;
}

// K1 with the (lanes per chain, coordinates per lane) shape params asks for
// (library default for n_dim when lanes_per_chain is 0)
int dispatch_local(const LocalArgs& a, const FmcLocalParams* params, cudaStream_t st);
int launch_local_mala(const LocalArgs& a, Shape sh, cudaStream_t st);
int launch_local_hmc(const LocalArgs& a, Shape sh, cudaStream_t st);
int launch_local_grw(const LocalArgs& a, Shape sh, cudaStream_t st);
int check_target(const FmcTarget* t);

}  // namespace fmc
