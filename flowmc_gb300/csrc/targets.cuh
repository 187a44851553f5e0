// targets.cuh -- registered target log-densities with hand-written adjoints.
//
// The reference takes an arbitrary JAX callable `logpdf(x, data)` and
// differentiates it with jax.value_and_grad (resource/kernel/MALA.py:59,
// resource/kernel/HMC.py:73-78). A fused device kernel cannot run Python, so
// the sampler is given a target descriptor (FmcTarget) and evaluates the
// value and its analytic gradient here.
//
// Work split: a chain is owned by a group of G lanes; lane `gl` holds the V
// consecutive coordinates j = gl*V + v (v < V) of the position. Coordinates
// j >= n_dim are padding: they hold 0, contribute 0 and get gradient 0.
// Reductions over coordinates are butterfly shuffles inside the group, so
// every lane of the group ends with the bitwise-same value.
#pragma once
#include "common.cuh"

namespace fmc {

constexpr int kMaxMixtureComponents = 16;

template <int V>
struct Vec { float v[V]; };

__device__ __forceinline__ float ldg_or(const float* p, int64_t i, float dflt) {
  return p ? __ldg(p + i) : dflt;
}

// The V entries of this lane's coordinates from one row of a shared-memory
// table (a lane's coordinates are fixed for the whole kernel); padding
// coordinates read 0. float4 loads when the rows are 16-byte aligned.
template <int V>
__device__ __forceinline__ void tab_row(const float* row, int gl, int d, float (&out)[V]) {
  const int j0 = gl * V;
  if constexpr (V % 4 == 0) {
    if ((d & 3) == 0) {
#pragma unroll
      for (int q = 0; q < V; q += 4) {
        // d % 4 == 0: a 4-coordinate chunk is either wholly inside the row or wholly padding
        const float4 t =
            (j0 + q < d) ? *reinterpret_cast<const float4*>(row + j0 + q) : make_float4(0.f, 0.f, 0.f, 0.f);
        out[q] = t.x; out[q + 1] = t.y; out[q + 2] = t.z; out[q + 3] = t.w;
      }
      return;
    }
  }
#pragma unroll
  for (int v = 0; v < V; ++v) out[v] = (j0 + v < d) ? row[j0 + v] : 0.f;
}

// Shared-memory copy of the diagonal-Gaussian / mixture tables: means
// [K * d] then inverse variances [K * d] (missing tables get 0 and 1).
__device__ __forceinline__ int target_table_floats(const FmcTarget& t) {
  const int K = (t.kind == FMC_TARGET_GAUSS_MIXTURE) ? t.n_comp : 1;
  return 2 * K * t.n_dim;
}
__device__ __forceinline__ void stage_target_table(const FmcTarget& t, float* tab) {
  const int n = target_table_floats(t) / 2;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    tab[i] = t.mean ? __ldg(t.mean + i) : 0.f;
    tab[n + i] = t.inv_var ? __ldg(t.inv_var + i) : 1.f;
  }
}

// --------------------------------------------------------------- diag Gaussian
// tab: the shared-memory table (stage_target_table) or NULL for global loads
template <int G, int V, bool GRAD>
__device__ __forceinline__ float tg_diag_gaussian(const FmcTarget& t, const float (&x)[V],
                                                  float (&g)[V], int gl, const float* tab) {
  const int d = t.n_dim;
  float s = 0.f;
  if (tab != nullptr) {
    float mu[V], iv[V];
    tab_row<V>(tab, gl, d, mu);
    tab_row<V>(tab + d, gl, d, iv);   // 0 on padding coordinates: no contribution
#pragma unroll
    for (int v = 0; v < V; ++v) {
      const float dx = x[v] - mu[v];
      s += dx * dx * iv[v];
      if (GRAD) g[v] = -dx * iv[v];
    }
    return -0.5f * group_sum<G>(s) + t.scalars[0];
  }
#pragma unroll
  for (int v = 0; v < V; ++v) {
    const int j = gl * V + v;
    if (j < d) {
      const float dx = x[v] - ldg_or(t.mean, j, 0.f);
      const float iv = ldg_or(t.inv_var, j, 1.f);
      s += dx * dx * iv;
      if (GRAD) g[v] = -dx * iv;
    } else if (GRAD) {
      g[v] = 0.f;
    }
  }
  return -0.5f * group_sum<G>(s) + t.scalars[0];
}

// --------------------------------------------------------------- dual moon
// log p = -0.5((|x| - s0)/s1)^2 + logsumexp(-0.5((x0 + s2)/s3)^2, -0.5((x0 - s2)/s3)^2)
template <int G, int V, bool GRAD>
__device__ __forceinline__ float tg_dual_moon(const FmcTarget& t, const float (&x)[V],
                                              float (&g)[V], int gl) {
  const int d = t.n_dim;
  const float s0 = t.scalars[0], s1 = t.scalars[1], s2 = t.scalars[2], s3 = t.scalars[3];
  float r2 = 0.f;
#pragma unroll
  for (int v = 0; v < V; ++v) r2 += x[v] * x[v];  // padding holds 0
  r2 = group_sum<G>(r2);
  const float r = sqrtf(r2);
  const float tt = (r - s0) / s1;
  const float x0 = group_bcast<G>(x[0], 0);
  const float za = (x0 + s2) / s3, zb = (x0 - s2) / s3;
  const float a = -0.5f * za * za, b = -0.5f * zb * zb;
  const float m = fmaxf(a, b);
  const float lse = m + log1pf(expf(-fabsf(a - b)));
  if (GRAD) {
    const float cr = -(tt / s1) / r;
#pragma unroll
    for (int v = 0; v < V; ++v) {
      const int j = gl * V + v;
      g[v] = (j < d) ? cr * x[v] : 0.f;
    }
    if (gl == 0) {
      const float wa = expf(a - lse), wb = expf(b - lse);
      g[0] += wa * (-za / s3) + wb * (-zb / s3);
    }
  }
  return -0.5f * tt * tt + lse;
}

// --------------------------------------------------------------- Gaussian mixture
// log p = logsumexp_k( log_w[k] - 0.5 sum_j (x_j - mean[k,j])^2 inv_var[k,j] )
// One pass over the components with an online log-sum-exp: running max m,
// running sum S = sum_k exp(e_k - m) and the running weighted gradient
// Gr = sum_k exp(e_k - m) * (-(x - mean_k) inv_var_k), rescaled whenever m
// grows; at the end lp = m + log S and grad = Gr / S. No per-component
// arrays, so the loop stays rolled and register use stays flat in K.
template <int G, int V, bool GRAD>
__device__ __forceinline__ float tg_mixture(const FmcTarget& t, const float (&x)[V],
                                            float (&g)[V], int gl, const float* tab) {
  const int d = t.n_dim, K = t.n_comp;
  float m = -INFINITY, S = 0.f;
  float Gr[V];
#pragma unroll
  for (int v = 0; v < V; ++v) Gr[v] = 0.f;
#pragma unroll 1
  for (int k = 0; k < K; ++k) {
    float q = 0.f;
    float gk[V];
    if (tab != nullptr) {
      float mu[V], iv[V];
      tab_row<V>(tab + k * d, gl, d, mu);
      tab_row<V>(tab + (K + k) * d, gl, d, iv);   // 0 on padding coordinates
#pragma unroll
      for (int v = 0; v < V; ++v) {
        const float dx = x[v] - mu[v];
        q += dx * dx * iv[v];
        gk[v] = -dx * iv[v];
      }
    } else {
#pragma unroll
      for (int v = 0; v < V; ++v) {
        const int j = gl * V + v;
        gk[v] = 0.f;
        if (j < d) {
          const float dx = x[v] - ldg_or(t.mean, (int64_t)k * d + j, 0.f);
          const float iv = ldg_or(t.inv_var, (int64_t)k * d + j, 1.f);
          q += dx * dx * iv;
          gk[v] = -dx * iv;
        }
      }
    }
    const float e = ldg_or(t.log_w, k, 0.f) - 0.5f * group_sum<G>(q);
    if (e > m) {
      const float r = expf(m - e);   // 0 on the first component (m = -inf)
      S = S * r + 1.f;
      if (GRAD) {
#pragma unroll
        for (int v = 0; v < V; ++v) Gr[v] = Gr[v] * r + gk[v];
      }
      m = e;
    } else {
      const float w = expf(e - m);
      S += w;
      if (GRAD) {
#pragma unroll
        for (int v = 0; v < V; ++v) Gr[v] += w * gk[v];
      }
    }
  }
  if (GRAD) {
    const float inv = 1.f / S;
#pragma unroll
    for (int v = 0; v < V; ++v) g[v] = Gr[v] * inv;
  }
  return m + logf(S);
}

// --------------------------------------------------------------- Rosenbrock chain
// log p = -sum_{i=0}^{d-2} [ (s1 - x_i)^2 / s0 + s2 (x_{i+1} - x_i^2)^2 ]
template <int G, int V, bool GRAD>
__device__ __forceinline__ float tg_rosenbrock(const FmcTarget& t, const float (&x)[V],
                                               float (&g)[V], int gl) {
  const int d = t.n_dim;
  const float s0 = t.scalars[0], s1 = t.scalars[1], s2 = t.scalars[2];
  // neighbours across the lane boundary
  const float next_first = __shfl_down_sync(0xffffffffu, x[0], 1, G);   // x_{gl*V+V}
  const float prev_last = __shfl_up_sync(0xffffffffu, x[V - 1], 1, G);  // x_{gl*V-1}
  float s = 0.f;
#pragma unroll
  for (int v = 0; v < V; ++v) {
    const int j = gl * V + v;
    const float xn = (v + 1 < V) ? x[v + 1] : next_first;
    const float xp = (v > 0) ? x[v - 1] : prev_last;
    const bool has_next = (j + 1 < d);
    const bool has_prev = (j >= 1) && (j < d);
    const float a = s1 - x[v];
    const float b = xn - x[v] * x[v];
    if (has_next) s += a * a / s0 + s2 * b * b;
    if (GRAD) {
      float gv = 0.f;
      if (has_next) gv += 2.f * a / s0 + 4.f * s2 * x[v] * b;
      if (has_prev) gv -= 2.f * s2 * (x[v] - xp * xp);
      g[v] = gv;
    }
  }
  return -group_sum<G>(s);
}

// --------------------------------------------------------------- dense Gaussian
// log p = -0.5 (x-m)^T P (x-m) + scalars[0], P symmetric (the host symmetrises).
// The group stages dx in shared memory (`stage`, n_dim floats per group).
template <int G, int V, bool GRAD>
__device__ __forceinline__ float tg_dense_gaussian(const FmcTarget& t, const float (&x)[V],
                                                   float (&g)[V], int gl, float* stage) {
  const int d = t.n_dim;
  float dx[V];
#pragma unroll
  for (int v = 0; v < V; ++v) {
    const int j = gl * V + v;
    dx[v] = (j < d) ? x[v] - ldg_or(t.mean, j, 0.f) : 0.f;
    if (j < d) stage[j] = dx[v];
  }
  __syncwarp();
  float acc[V];
#pragma unroll
  for (int v = 0; v < V; ++v) acc[v] = 0.f;
  for (int k = 0; k < d; ++k) {
    const float dk = stage[k];
    const float* row = t.precision + (int64_t)k * d;
#pragma unroll
    for (int v = 0; v < V; ++v) {
      const int j = gl * V + v;
      if (j < d) acc[v] += __ldg(row + j) * dk;  // P[k, j] = P[j, k]
    }
  }
  __syncwarp();
  float s = 0.f;
#pragma unroll
  for (int v = 0; v < V; ++v) {
    s += dx[v] * acc[v];
    if (GRAD) g[v] = -acc[v];
  }
  return -0.5f * group_sum<G>(s) + t.scalars[0];
}

// stage: the dense Gaussian's per-group scratch (n_dim floats), or for the
// diagonal Gaussian and the mixture the block's shared-memory table copy
// (stage_target_table; NULL = read the tables from global memory)
template <int TGT, int G, int V, bool GRAD>
__device__ __forceinline__ float target_eval(const FmcTarget& t, const float (&x)[V],
                                             float (&g)[V], int gl, float* stage) {
  if constexpr (TGT == FMC_TARGET_DIAG_GAUSSIAN) return tg_diag_gaussian<G, V, GRAD>(t, x, g, gl, stage);
  else if constexpr (TGT == FMC_TARGET_DUAL_MOON) return tg_dual_moon<G, V, GRAD>(t, x, g, gl);
  else if constexpr (TGT == FMC_TARGET_GAUSS_MIXTURE) return tg_mixture<G, V, GRAD>(t, x, g, gl, stage);
  else if constexpr (TGT == FMC_TARGET_ROSENBROCK) return tg_rosenbrock<G, V, GRAD>(t, x, g, gl);
  else return tg_dense_gaussian<G, V, GRAD>(t, x, g, gl, stage);
}

}  // namespace fmc
