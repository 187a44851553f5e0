// tc_spline.cu -- the last conditioner Linear fused with the rational-quadratic
// spline (forward or inverse) on the tensor cores.
//
// For one coupling layer, rows [0, M) of the previous tanh activation A (bf16)
// are multiplied by the last Linear's weights, re-packed in groups: group g
// holds the DG = floor(256 / P) transformed coordinates t = g*DG .. g*DG+DG-1,
// each as its P = 3K+1 consecutive weight rows, padded to BN rows (a multiple
// of 16). The accumulator of a (128-row, group) tile therefore holds, for
// every row, the complete raw spline parameters of DG coordinates. The
// epilogue threads (one accumulator row each) add the bias, build the knots,
// evaluate the spline (rqSpline.py:42-239) on x = xa[row, 2t + tpar], write
// the result back into xa and leave the row's log-determinant partial sum in
// ldp[row, 2g + half]. The conditioner outputs never reach global memory.
//
// Structure as k_tc_gemm (tc_gemm.cuh): persistent CTAs, TMA producer warp,
// MMA warp, two TMEM accumulators; here kSplineEpiPerQuarter epilogue warps
// per TMEM lane quarter, warp h of a quarter taking coordinates h, h + E, ...
// of the group. Only the bin that holds each input is built
// (rqs_apply_fast). All waits are bounded.
#include "flow.cuh"
#include "tc_gemm.cuh"

namespace fmc {
namespace tc {

constexpr int kSplEpiWarps = 4 * kSplineEpiPerQuarter;
constexpr int kSplThreads = 64 + 32 * kSplEpiWarps;

template <int K>
struct SplineTile {
  static constexpr int P = 3 * K + 1;
  static constexpr int DG = 256 / P;
  static constexpr int BN = ((DG * P + 15) / 16) * 16;
};

// N consecutive accumulator columns of this thread's lane; every register is
// pinned after the wait so no use can be scheduled before the data arrive
template <int N>
__device__ __forceinline__ void tmem_ld_cols(uint32_t taddr, float (&v)[N]) {
  uint32_t r[N];
#pragma unroll
  for (int i = 0; i < N; ++i)
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x1.b32 {%0}, [%1];" : "=r"(r[i]) : "r"(taddr + (uint32_t)i));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < N; ++i) {
    asm volatile("" : "+r"(r[i]));
    v[i] = __uint_as_float(r[i]);
  }
}

template <int KB, bool INV, int STAGES>
__global__ void __launch_bounds__(kSplThreads, 1)
    k_tc_spline(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, int M, int n_groups,
                int nt, int K, const float* __restrict__ bias, float* __restrict__ xa, int d, int tpar,
                float* __restrict__ ldp, SplineCfg cfg, int* err) {
  using T = SplineTile<KB>;
  constexpr int P = T::P, DG = T::DG, BN = T::BN;
  using S = Smem<BN, STAGES>;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* base = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(base + STAGES * S::STAGE_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* acc_full = empty + STAGES;
  uint64_t* acc_empty = acc_full + 2;
  uint64_t* mma_done = acc_empty + 2;
  uint32_t* tmem_slot = (uint32_t*)(mma_done + 1);
  volatile int* abort_flag = (volatile int*)(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nk = (K + BK - 1) / BK;
  const int m_tiles = (M + BM - 1) / BM;
  const int tiles = m_tiles * n_groups;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], kSplEpiWarps);
    }
    mbar_init(mma_done, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(512));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      uint32_t it = 0;
      for (int t = blockIdx.x; t < tiles && !*abort_flag; t += gridDim.x) {
        const int m0 = (t / n_groups) * BM, n0 = (t % n_groups) * BN;
        for (int k = 0; k < nk; ++k, ++it) {
          const int s = it % STAGES;
          const uint32_t ph = (it / STAGES) & 1u;
          if (it >= (uint32_t)STAGES && !mbar_wait(&empty[s], ph ^ 1u)) {
            *abort_flag = 1;
            break;
          }
          if (*abort_flag) break;
          uint8_t* sa = base + s * S::STAGE_BYTES;
          uint8_t* sb = sa + S::A_BYTES;
          mbar_expect_tx(&full[s], S::STAGE_BYTES);
          tma_load_2d(sa, &tmA, &full[s], k * BK, m0);
          tma_load_2d(sb, &tmB, &full[s], k * BK, n0);
        }
      }
      if (*abort_flag) {
        for (uint32_t j = it > (uint32_t)STAGES ? it - STAGES : 0; j < it; ++j)
          mbar_wait(&full[j % STAGES], (j / STAGES) & 1u);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t idesc = idesc_bf16_f32(BN);
      uint32_t it = 0;
      int local = 0;
      for (int t = blockIdx.x; t < tiles && !*abort_flag; t += gridDim.x, ++local) {
        const int b = local & 1, use = local >> 1;
        if (use > 0 && !mbar_wait(&acc_empty[b], (uint32_t)(use - 1) & 1u)) {
          *abort_flag = 1;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t dcol = tmem + (uint32_t)(b * 256);
        bool stop = false;
        for (int k = 0; k < nk; ++k, ++it) {
          const int s = it % STAGES;
          const uint32_t ph = (it / STAGES) & 1u;
          if (!mbar_wait(&full[s], ph) || *abort_flag) {
            *abort_flag = 1;
            stop = true;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint8_t* sa = base + s * S::STAGE_BYTES;
          const uint8_t* sb = sa + S::A_BYTES;
          const uint64_t da = smem_desc_sw128(sa), db = smem_desc_sw128(sb);
#pragma unroll
          for (int kk = 0; kk < BK / 16; ++kk)
            mma_bf16(dcol, da + (uint64_t)(kk * 2), db + (uint64_t)(kk * 2), idesc, (k > 0 || kk > 0) ? 1u : 0u);
          mma_commit(&empty[s]);
        }
        if (stop) break;
        mma_commit(&acc_full[b]);
      }
      mma_commit(mma_done);
    }
  } else {
    constexpr int E = kSplineEpiPerQuarter;
    const int ew = warp - 2;
    const int q = warp & 3;          // TMEM lane quarter
    const int half = ew >> 2;        // coordinates half, half + E, ... of the group
    const int row = q * 32 + lane;
    int local = 0;
    for (int t = blockIdx.x; t < tiles; t += gridDim.x, ++local) {
      const int b = local & 1, use = local >> 1;
      const int m0 = (t / n_groups) * BM, g = t % n_groups;
      const int gm = m0 + row;
      if (*abort_flag || !mbar_wait(&acc_full[b], (uint32_t)use & 1u)) {
        *abort_flag = 1;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t tb = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * 256);
      float ldsum = 0.f;
#pragma unroll 1
      for (int u = half; u < DG; u += E) {
        const int tcoord = g * DG + u;
        if (tcoord >= nt) break;
        float raw[P];
        tmem_ld_cols<P>(tb + (uint32_t)(u * P), raw);   // warp-collective: every lane loads
        if (gm < M) {
          float* xp = xa + (int64_t)gm * d + 2 * tcoord + tpar;
          const float xv = *xp;
          const float* bb = bias + (int64_t)tcoord * P;
#pragma unroll
          for (int p = 0; p < P; ++p) raw[p] += __ldg(bb + p);
          float y, l;
          rqs_apply_fast<KB, INV>(raw, xv, cfg, y, l);
          *xp = y;
          ldsum += l;
        }
      }
      if (gm < M) ldp[(int64_t)gm * (E * n_groups) + E * g + half] = ldsum;
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(&acc_empty[b]);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    if (lane == 0) mbar_wait(mma_done, 0);
    __syncwarp();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
  }
  if (threadIdx.x == 0 && *abort_flag) atomicExch(err, 1);
}

}  // namespace tc

// ld[r] += sum of the row's kSplineEpiPerQuarter * n_groups partials (fixed order)
__global__ void k_ld_reduce(const float* __restrict__ ldp, int n_part, int64_t m, float* __restrict__ ld) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < m; r += (int64_t)gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int j = 0; j < n_part; ++j) s += ldp[r * n_part + j];
    ld[r] += s;
  }
}

int tc_error_word(int** out);
int make_tma_map_bf16(CUtensorMap* m, const void* base, int64_t inner, int64_t outer, int64_t ld, int box_outer);

int spline_groups(int K_bins, int nt, int* dg, int* bn) {
  const int P = 3 * K_bins + 1;
  const int DG = 256 / P;
  *dg = DG;
  *bn = ((DG * P + 15) / 16) * 16;
  return (nt + DG - 1) / DG;
}

template <int KB, bool INV>
static int launch_spl(cudaStream_t st, const CUtensorMap& ma, const CUtensorMap& mb, int64_t M, int n_groups, int nt,
                      int K, const float* bias, float* xa, int d, int tpar, float* ldp, SplineCfg cfg) {
  constexpr int STAGES = 4;
  using S = tc::Smem<tc::SplineTile<KB>::BN, STAGES>;
  auto kern = tc::k_tc_spline<KB, INV, STAGES>;
  static bool attr = false;
  if (!attr) {
    FMC_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, S::TOTAL));
    attr = true;
  }
  int* err = nullptr;
  int rc = tc_error_word(&err);
  if (rc) return rc;
  const int64_t tiles = (M + tc::BM - 1) / tc::BM * n_groups;
  const int64_t grid = tiles < sm_count() ? tiles : sm_count();
  kern<<<(unsigned)grid, tc::kSplThreads, S::TOTAL, st>>>(ma, mb, (int)M, n_groups, nt, K, bias, xa, d, tpar, ldp,
                                                           cfg, err);
  FMC_LAUNCH_CHECK();
  return FMC_OK;
}

// The last Linear of layer l fused with its spline: A = the last tanh
// activation (bf16 [rows_a, K]), Bg = the grouped weights, xa updated in place,
// ld[r] accumulated.
int tc_linear_spline(cudaStream_t st, const FlowGeom& g, const FmcFlow* f, int l, const uint16_t* A, int64_t M,
                     int64_t rows_a, bool inverse, float* xa, float* ld, float* ldp) {
  const int nt = g.nt(l);
  int dg, bn;
  const int n_groups = spline_groups(g.K, nt, &dg, &bn);
  const int Kd = g.w16_cols(l, g.nh);
  const uint16_t* Bg = f->theta_bf16 + g.w16g_off[l];
  const float* bias = f->theta + g.layer_off[l] + g.lin_b(l, g.nh);
  CUtensorMap ma, mb;
  int rc = make_tma_map_bf16(&ma, A, Kd, rows_a, Kd, tc::BM);
  if (rc) return rc;
  if ((rc = make_tma_map_bf16(&mb, Bg, Kd, (int64_t)n_groups * bn, Kd, bn))) return rc;
#define SPL_CASE(k)                                                                                              \
  if (g.K == k) {                                                                                                \
    rc = inverse ? launch_spl<k, true>(st, ma, mb, M, n_groups, nt, Kd, bias, xa, g.d, g.tpar(l), ldp, g.cfg)    \
                 : launch_spl<k, false>(st, ma, mb, M, n_groups, nt, Kd, bias, xa, g.d, g.tpar(l), ldp, g.cfg);  \
  } else
  SPL_CASE(2) SPL_CASE(3) SPL_CASE(4) SPL_CASE(5) SPL_CASE(6) SPL_CASE(8) SPL_CASE(10) SPL_CASE(12) SPL_CASE(16) {
    set_error("n_bins=%d is not instantiated for the fused spline", g.K);
    return FMC_ERR_UNSUPPORTED;
  }
#undef SPL_CASE
  if (rc) return rc;
  int64_t blocks = (M + 255) / 256;
  if (blocks > (int64_t)sm_count() * 8) blocks = (int64_t)sm_count() * 8;
  k_ld_reduce<<<(int)(blocks < 1 ? 1 : blocks), 256, 0, st>>>(ldp, kSplineEpiPerQuarter * n_groups, M, ld);
  FMC_LAUNCH_CHECK();
  return FMC_OK;
}

}  // namespace fmc
