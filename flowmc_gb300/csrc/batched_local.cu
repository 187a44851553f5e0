// batched_local.cu -- many independent dense-Gaussian targets of uneven
// dimension sampled in ONE persistent launch (MALA or HMC).
//
// Work items are tiles of up to 32 chains of one target; CTAs pull items from
// an atomic counter (a persistent scheduler: long items never leave SMs idle
// behind short ones) and run all n_steps of their tile before taking the next.
// A tile keeps its positions, gradients and log-densities in shared memory
// for the whole run. The gradient of log p = -0.5 dx^T P dx (dx = x - mean,
// P symmetric) is a [32 x d] x [d x d] product per evaluation: each thread owns
// 8 chains x 4 coordinates of the output and streams P rows from L2 (one P per
// target serves all its tiles), dx comes from shared memory.
//
// Step semantics are those of fmc_local_steps (MALA.py:26-89, HMC.py:98-151
// with an identity mass matrix); the output of target t is written to its own
// buffers [n_chains_t, buf_len, d_t] at the clamped cursor.
#include <vector>
#include "local_steps.cuh"

namespace fmc {

constexpr int kBT = 32;          // chains per tile
constexpr int kBThreads = 256;   // 64 column groups x 4 chain groups
constexpr int kBDMax = 256;

struct BatchTarget {
  const float* precision;   // [d, d]
  const float* mean;        // [d] or NULL
  float const_term;
  int d;
  int n_chains;
  int chain_offset;         // first row of this target in x0 / x_last / lp_last ([sum C, 256])
  float* out_pos;           // [n_chains, buf_len, d]
  float* out_logp;          // [n_chains, buf_len]
  float* out_acc;
  float step;
  const float* noise;       // [n_chains, n_steps, d] explicit normals or NULL
  const float* unif;        // [n_chains, n_steps] explicit uniforms or NULL
};

struct BatchArgs {
  const BatchTarget* targets;
  const int32_t* item_target;   // [n_items]
  const int32_t* item_chain0;   // [n_items]
  int n_items;
  int* next_item;               // scheduler counter (zeroed before the launch)
  int kind, n_leapfrog, S, thin;
  int64_t buf_len, start;
  Rng rng;
  const float* x0;              // [sum C, 256] (row stride 256)
  float* x_last;                // [sum C, 256]
  float* lp_last;               // [sum C]
};

// Y[c][j] = sum_k DX[c][k] P[k][j] for the tile; also lp_c = -0.5 sum_j DX Y + const.
// Thread (cg, jg): chains cg*8..cg*8+7, columns jg*4..jg*4+3. The k loop runs
// in chunks of 4 rows of P with the next two chunks' P values already in
// registers (the rows stream from L2 with only 8 warps per SM to hide their
// latency); the 8 chains' dx for a chunk are one float4 shared-memory load each.
__device__ __forceinline__ void load_p4(const float* __restrict__ P, int d, int k0, int j0, float (&p)[4][4]) {
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int k = k0 + r;
    const float* row = P + (int64_t)k * d + j0;
#pragma unroll
    for (int u = 0; u < 4; ++u) p[r][u] = (k < d && j0 + u < d) ? __ldg(row + u) : 0.f;
  }
}

__device__ void dense_eval(const BatchTarget& T, const float* X, float* DX, float* G, float* lp, float* red) {
  const int tid = threadIdx.x, jg = tid & 63, cg = tid >> 6;
  const int d = T.d;
  {
    // dx = x - mean, zero beyond d up to the next multiple of 4 (read by the float4 loads)
    const int c = tid >> 3, sub = tid & 7;
    const int d4 = (d + 3) & ~3;
    for (int j = sub; j < d4; j += 8)
      DX[c * kBDMax + j] = (j < d) ? X[c * kBDMax + j] - (T.mean ? __ldg(T.mean + j) : 0.f) : 0.f;
  }
  __syncthreads();
  float acc[8][4] = {};
  const int j0 = jg * 4;
  if (j0 < d) {
    // three register buffers in fixed roles over an unrolled group of three
    // chunks, so no buffer is ever copied; rows >= d read as zeros
    float pa[4][4], pb[4][4], pc[4][4];
    auto fma_chunk = [&](int k0, const float (&p)[4][4]) {
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        const float4 xv = *reinterpret_cast<const float4*>(DX + (cg * 8 + c) * kBDMax + k0);
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          acc[c][u] = fmaf(xv.x, p[0][u], acc[c][u]);
          acc[c][u] = fmaf(xv.y, p[1][u], acc[c][u]);
          acc[c][u] = fmaf(xv.z, p[2][u], acc[c][u]);
          acc[c][u] = fmaf(xv.w, p[3][u], acc[c][u]);
        }
      }
    };
    load_p4(T.precision, d, 0, j0, pa);
    load_p4(T.precision, d, 4, j0, pb);
    for (int k0 = 0; k0 < d; k0 += 12) {
      load_p4(T.precision, d, k0 + 8, j0, pc);
      fma_chunk(k0, pa);
      if (k0 + 4 >= d) break;
      load_p4(T.precision, d, k0 + 12, j0, pa);
      fma_chunk(k0 + 4, pb);
      if (k0 + 8 >= d) break;
      load_p4(T.precision, d, k0 + 16, j0, pb);
      fma_chunk(k0 + 8, pc);
    }
  }
  // gradient -P dx and the per-chain partial of dx . P dx
  float part[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    part[c] = 0.f;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int j = j0 + u;
      if (j < d) {
        G[(cg * 8 + c) * kBDMax + j] = -acc[c][u];
        part[c] += DX[(cg * 8 + c) * kBDMax + j] * acc[c][u];
      }
    }
  }
  // reduce over the 64 column groups: warp shuffles then shared memory
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    float v = part[c];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((tid & 31) == 0) red[(cg * 8 + c) * 2 + ((tid >> 5) & 1)] = v;
  }
  __syncthreads();
  if (tid < kBT) lp[tid] = -0.5f * (red[tid * 2] + red[tid * 2 + 1]) + T.const_term;
  __syncthreads();
}

// Elementwise passes over a tile use the same mapping: 8 threads per chain
// (256 threads = 32 chains), thread tid on chain tid >> 3 and coordinates
// (tid & 7) + 8i.
// per-chain sum over j < d of f(c, j) in a fixed order: 8 threads per chain
// (256 threads = 32 chains), strided over j, then a 3-level shuffle
template <typename F>
__device__ __forceinline__ float chain_sum(int d, F f) {
  const int tid = threadIdx.x, c = tid >> 3, sub = tid & 7;
  float v = 0.f;
  for (int j = sub; j < d; j += 8) v += f(c, j);
  v += __shfl_xor_sync(0xffffffffu, v, 1);
  v += __shfl_xor_sync(0xffffffffu, v, 2);
  v += __shfl_xor_sync(0xffffffffu, v, 4);
  return v;
}

// normal for (chain c of T, step s, coordinate j): explicit or Philox
__device__ __forceinline__ float draw_normal(const BatchArgs& a, const Rng& rng, const BatchTarget& T, int c, int s,
                                             int j) {
  if (T.noise) return (c < T.n_chains) ? __ldg(T.noise + ((int64_t)c * a.S + s) * T.d + j) : 0.f;
  const u32x4 r = rng.draw((uint64_t)(T.chain_offset + c), (uint64_t)s, (uint32_t)(j >> 1), RNG_TAG_LOCAL_NORMAL);
  float z0, z1;
  box_muller(r.x, r.y, z0, z1);
  return (j & 1) ? z1 : z0;
}

__global__ void __launch_bounds__(kBThreads) k_batched_dense(const BatchArgs a) {
  extern __shared__ float sm[];
  const Rng rng = a.rng.at_epoch();
  float* X = sm;                      // [32][256] current positions
  float* Gx = X + kBT * kBDMax;       // gradient at X
  float* Y = Gx + kBT * kBDMax;       // proposal / leapfrog position
  float* Gy = Y + kBT * kBDMax;       // gradient at Y
  float* DX = Gy + kBT * kBDMax;      // scratch dx
  float* Pm = DX + kBT * kBDMax;      // HMC momentum
  float* lpx = Pm + kBT * kBDMax;     // [32]
  float* lpy = lpx + kBT;
  float* red = lpy + kBT;             // [64]
  float* sA = red + 2 * kBT;          // [32] per-chain sums
  float* sB = sA + kBT;
  float* xr_lp = sB + kBT;            // [32] log-density of the last written row
  __shared__ int item_s;
  const int tid = threadIdx.x;

  for (;;) {
    if (tid == 0) item_s = atomicAdd(a.next_item, 1);
    __syncthreads();
    const int item = item_s;
    __syncthreads();
    if (item >= a.n_items) break;
    const BatchTarget T = a.targets[a.item_target[item]];
    const int c0 = a.item_chain0[item];
    const int nc = min(kBT, T.n_chains - c0);
    const int d = T.d;
    const float dt = T.step;
    for (int e = tid; e < kBT * kBDMax; e += kBThreads) {
      const int c = e / kBDMax, j = e - c * kBDMax;
      X[e] = (c < nc && j < d) ? a.x0[(int64_t)(T.chain_offset + c0 + c) * kBDMax + j] : 0.f;
    }
    __syncthreads();
    dense_eval(T, X, DX, Gx, lpx, red);
    for (int s = 0; s < a.S; ++s) {
      // ---- proposal (MALA) or leapfrog trajectory (HMC) into Y / Gy / lpy
      if (a.kind == FMC_KERNEL_MALA) {
        const float dt2 = dt * dt;
        for (int j = tid & 7, c = tid >> 3; j < d; j += 8) {
          const float xi = draw_normal(a, rng, T, c0 + c, s, j);
          const int i = c * kBDMax + j;
          Y[i] = (X[i] + dt2 * Gx[i] / 2.0f) + dt * xi;
        }
        __syncthreads();
        dense_eval(T, Y, DX, Gy, lpy, red);
        // |prop - mean0|^2 and |x - mean1|^2 per chain
        const float va = chain_sum(d, [&](int c, int j) {
          const int i = c * kBDMax + j;
          const float ea = Y[i] - (X[i] + dt2 * Gx[i] / 2.0f);
          return ea * ea;
        });
        const float vb = chain_sum(d, [&](int c, int j) {
          const int i = c * kBDMax + j;
          const float eb = X[i] - (Y[i] + dt2 * Gy[i] / 2.0f);
          return eb * eb;
        });
        if ((tid & 7) == 0) { sA[tid >> 3] = va; sB[tid >> 3] = vb; }
        __syncthreads();
      } else {
        for (int j = tid & 7, c = tid >> 3; j < d; j += 8) {
          const int i = c * kBDMax + j;
          Pm[i] = draw_normal(a, rng, T, c0 + c, s, j);
          Y[i] = X[i];
          Gy[i] = Gx[i];
        }
        __syncthreads();
        {
          const float v0 = chain_sum(d, [&](int c, int j) {
            const float p = Pm[c * kBDMax + j];
            return p * p;
          });
          if ((tid & 7) == 0) sA[tid >> 3] = v0;
        }
        __syncthreads();
        // row 0: half kick with the gradient at x
        for (int j = tid & 7, c = tid >> 3; j < d; j += 8) {
          const int i = c * kBDMax + j;
          Pm[i] = Pm[i] + (dt * 0.5f) * Gy[i];
        }
        __syncthreads();
        for (int r = 1; r <= a.n_leapfrog + 1; ++r) {
          const float ek = (r == a.n_leapfrog + 1) ? dt * 0.5f : dt;
          for (int j = tid & 7, c = tid >> 3; j < d; j += 8) {
            const int i = c * kBDMax + j;
            Y[i] = Y[i] + dt * Pm[i];
          }
          __syncthreads();
          dense_eval(T, Y, DX, Gy, lpy, red);
          for (int j = tid & 7, c = tid >> 3; j < d; j += 8) {
            const int i = c * kBDMax + j;
            Pm[i] = Pm[i] + ek * Gy[i];
          }
          __syncthreads();
        }
        {
          const float v1 = chain_sum(d, [&](int c, int j) {
            const float p = Pm[c * kBDMax + j];
            return p * p;
          });
          if ((tid & 7) == 0) sB[tid >> 3] = v1;
        }
        __syncthreads();
      }
      // ---- accept per chain (float-float log-ratio), then commit
      __shared__ int acc_s[kBT];
      if (tid < kBT) {
        const int c = tid;
        const int64_t chain = T.chain_offset + c0 + c;
        float u;
        if (T.unif) u = (c < nc) ? __ldg(T.unif + (int64_t)(c0 + c) * a.S + s) : 1.f;
        else u = u32_to_unit(rng.draw((uint64_t)chain, (uint64_t)s, 0u, RNG_TAG_LOCAL_UNIFORM).x);
        const float logu = logf(u);
        ff ratio;
        if (a.kind == FMC_KERNEL_MALA) {
          const ff q = two_sum(sA[c], -sB[c]);
          ratio = ff_add(two_sum(lpy[c], -lpx[c]), ff_mul_f(q, 0.5f / (dt * dt)));
        } else {
          ratio = ff_add(two_sum(-lpx[c], 0.5f * sA[c]), ff_neg(two_sum(-lpy[c], 0.5f * sB[c])));
        }
        acc_s[c] = (c < nc) && f_lt_ff(logu, ratio) ? 1 : 0;
      }
      __syncthreads();
      for (int j = tid & 7, c = tid >> 3; j < d; j += 8) {
        if (acc_s[c]) {
          const int i = c * kBDMax + j;
          X[i] = Y[i];
          Gx[i] = Gy[i];
        }
      }
      if (tid < kBT && acc_s[tid]) lpx[tid] = lpy[tid];
      __syncthreads();
      if (s % a.thin == 0) {
        const int64_t row = a.start + s / a.thin;
        for (int j = tid & 7, c = tid >> 3; c < nc && j < d; j += 8) {
          __stcs(T.out_pos + ((int64_t)(c0 + c) * a.buf_len + row) * d + j, X[c * kBDMax + j]);
        }
        if (tid < nc) {
          __stcs(T.out_logp + (int64_t)(c0 + tid) * a.buf_len + row, lpx[tid]);
          __stcs(T.out_acc + (int64_t)(c0 + tid) * a.buf_len + row, acc_s[tid] ? 1.f : 0.f);
          xr_lp[tid] = lpx[tid];
        }
        for (int j = tid & 7, c = tid >> 3; c < nc && j < d; j += 8) {
          a.x_last[(int64_t)(T.chain_offset + c0 + c) * kBDMax + j] = X[c * kBDMax + j];
        }
      }
      __syncthreads();
    }
    if (tid < nc) a.lp_last[T.chain_offset + c0 + tid] = xr_lp[tid];
    __syncthreads();
  }
}

}  // namespace fmc

using namespace fmc;

extern "C" int fmc_batched_workspace_size(int32_t n_targets, int64_t total_chains, size_t* bytes) {
  FMC_CHECK_ARG(bytes && n_targets >= 1 && total_chains >= 1, "bad arguments");
  const int64_t items = total_chains / kBT + n_targets;
  *bytes = (size_t)(256 + n_targets * sizeof(BatchTarget) + 256 + items * 8 + 256);
  return FMC_OK;
}

extern "C" int fmc_batched_dense_local_steps(const FmcTarget* targets, int32_t n_targets, const int32_t* n_chains,
                                             const FmcLocalParams* params, const float* step_sizes,
                                             const float* x0, int32_t n_steps, int32_t thinning, uint64_t seed,
                                             uint64_t counter, const float* const* noise, const float* const* unif,
                                             float* const* out_pos, float* const* out_logp,
                                             float* const* out_acc, int64_t buf_len, int64_t cursor, float* x_last,
                                             float* lp_last, void* ws, size_t ws_bytes, void* stream) {
  FMC_CHECK_ARG(targets && n_chains && params && step_sizes && out_pos && out_logp && out_acc, "NULL host array");
  FMC_CHECK_ARG(n_targets >= 1, "n_targets < 1");
  FMC_CHECK_ARG(params->kind == FMC_KERNEL_MALA || params->kind == FMC_KERNEL_HMC,
                "batched dense targets run MALA or HMC");
  FMC_CHECK_ARG(params->kind != FMC_KERNEL_HMC || params->n_leapfrog >= 0, "n_leapfrog < 0");
  FMC_CHECK_ARG(n_steps >= 1 && thinning >= 1 && cursor >= 0, "bad step arguments");
  const int64_t n_rec = ((int64_t)n_steps + thinning - 1) / thinning;
  FMC_CHECK_ARG(n_rec <= buf_len, "update of %lld rows does not fit a buffer of %lld rows", (long long)n_rec,
                (long long)buf_len);
  FMC_CHECK_ARG(x0 && x_last && lp_last, "NULL device array");
  std::vector<BatchTarget> bt(n_targets);
  std::vector<int32_t> it, ic;
  int64_t off = 0;
  for (int t = 0; t < n_targets; ++t) {
    const FmcTarget& g = targets[t];
    FMC_CHECK_ARG(g.kind == FMC_TARGET_DENSE_GAUSSIAN, "target %d is not a dense Gaussian", t);
    FMC_CHECK_ARG(g.n_dim >= 1 && g.n_dim <= kBDMax, "target %d: n_dim %d outside [1, %d]", t, g.n_dim, kBDMax);
    FMC_CHECK_ARG(g.precision != nullptr, "target %d: no precision matrix", t);
    FMC_CHECK_ARG(n_chains[t] >= 1, "target %d: no chains", t);
    FMC_CHECK_ARG(out_pos[t] && out_logp[t] && out_acc[t], "target %d: NULL output buffer", t);
    bt[t] = BatchTarget{g.precision, g.mean, g.scalars[0], g.n_dim, n_chains[t], (int)off,
                        out_pos[t], out_logp[t], out_acc[t], step_sizes[t],
                        noise ? noise[t] : nullptr, unif ? unif[t] : nullptr};
    for (int c = 0; c < n_chains[t]; c += kBT) {
      it.push_back(t);
      ic.push_back(c);
    }
    off += n_chains[t];
  }
  size_t need = 0;
  fmc_batched_workspace_size(n_targets, off, &need);
  FMC_CHECK_ARG(ws && ws_bytes >= need, "workspace of %zu bytes < %zu needed", ws_bytes, need);
  cudaStream_t st = (cudaStream_t)stream;
  char* p = (char*)ws;
  int* next = (int*)p;
  p += 256;
  BatchTarget* dt = (BatchTarget*)p;
  p += (n_targets * sizeof(BatchTarget) + 255) / 256 * 256;
  int32_t* ditem_t = (int32_t*)p;
  int32_t* ditem_c = ditem_t + it.size();
  // the tables go up with the stream; copies from pageable memory are staged
  // before cudaMemcpyAsync returns, so the host vectors may go out of scope
  FMC_CUDA_TRY(cudaMemsetAsync(next, 0, sizeof(int), st));
  FMC_CUDA_TRY(cudaMemcpyAsync(dt, bt.data(), n_targets * sizeof(BatchTarget), cudaMemcpyHostToDevice, st));
  FMC_CUDA_TRY(cudaMemcpyAsync(ditem_t, it.data(), it.size() * 4, cudaMemcpyHostToDevice, st));
  FMC_CUDA_TRY(cudaMemcpyAsync(ditem_c, ic.data(), ic.size() * 4, cudaMemcpyHostToDevice, st));
  BatchArgs a{};
  a.targets = dt;
  a.item_target = ditem_t;
  a.item_chain0 = ditem_c;
  a.n_items = (int)it.size();
  a.next_item = next;
  a.kind = params->kind;
  a.n_leapfrog = params->n_leapfrog;
  a.S = n_steps;
  a.thin = thinning;
  a.buf_len = buf_len;
  a.start = cursor < buf_len - n_rec ? cursor : buf_len - n_rec;
  a.rng = Rng{(uint32_t)seed, (uint32_t)(seed >> 32), counter, rng_epoch()};
  a.x0 = x0;
  a.x_last = x_last;
  a.lp_last = lp_last;
  const size_t smem = (size_t)(6 * kBT * kBDMax + 6 * kBT + 2 * kBT) * sizeof(float);
  FMC_CUDA_TRY(cudaFuncSetAttribute(k_batched_dense, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  FMC_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batched_dense, kBThreads, smem));
  if (per_sm < 1) per_sm = 1;
  int64_t grid = (int64_t)sm_count() * per_sm;
  if (grid > a.n_items) grid = a.n_items;
  k_batched_dense<<<(int)grid, kBThreads, smem, st>>>(a);
  FMC_LAUNCH_CHECK();
  return FMC_OK;
}
