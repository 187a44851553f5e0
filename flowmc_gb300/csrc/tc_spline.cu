// tc_spline.cu -- the last conditioner Linear fused with the rational-quadratic
// spline on the tensor cores: the forward/inverse pass (inference and the
// training forward) and the spline adjoint (training backward).
//
// For one coupling layer, rows [0, M) of the previous tanh activation A (bf16)
// are multiplied by the last Linear's weights, re-packed in groups: group g
// holds the DG = floor(256 / P) transformed coordinates t = g*DG .. g*DG+DG-1,
// each as its P = 3K+1 consecutive weight rows, padded to BN rows (a multiple
// of 16). The accumulator of a (128-row, group) tile therefore holds, for
// every row, the complete raw spline parameters of DG coordinates, and the
// conditioner outputs never reach global memory.
//
//   k_tc_spline      epilogue: bias, knots of the selected bin only, the
//                    spline (rqSpline.py:42-239) on x = xa[row, 2t + tpar]
//                    written back into xa; per-row log-determinant partials
//                    into ldp[(E*g + h) * M + row] (one per group, g * M + row,
//                    with the x boxes); optionally the next coupling layer's
//                    ScalarAffine and its bf16 conditioning operand (fold)
//   k_tc_spline_bwd  epilogue: bias, knots, the spline adjoint of the
//                    selected bin (rqs_fwd_adjoint_fast) given
//                    dL/dy = gy[row, 2t + tpar] and dL/dlogdet = gld; dL/dx
//                    into gxa, dL/draw as bf16 staged in shared memory and
//                    stored by TMA in the padded layout [row, t*OPC + p]
//                    (read row-major by the input-gradient GEMM and MN-major
//                    by the weight-gradient GEMM), plus per-tile column sums
//                    for the bias gradient
//
// Both kernels are persistent (tile t = blockIdx.x, +gridDim.x, ...): warp 0
// issues the TMA loads of a STAGES-deep ring (stages of one or, for the
// forward/inverse kernel where K allows, two 64-wide K chunks), warp 1 owns
// the TMEM and issues tcgen05.mma into two accumulators (the epilogue of one tile overlaps the
// MMAs of the next), and kSplineEpiPerQuarter warps per TMEM lane quarter run
// the epilogue, warp h of a quarter taking coordinates h, h + E, ... of the
// group. Every mbarrier wait is bounded; on expiry the kernel raises the
// device error word, skips the remaining work, still frees its TMEM and
// returns.
#include "flow.cuh"
#include "tc_gemm.cuh"

namespace fmc {
namespace tc {

constexpr int kSplEpiWarps = 4 * kSplineEpiPerQuarter;
constexpr int kSplEpiThreads = 32 * kSplEpiWarps;
constexpr int kSplThreads = 64 + kSplEpiThreads;

template <int K>
struct SplineTile {
  static constexpr int P = 3 * K + 1;
  static constexpr int PPC = (P + 7) / 8 * 8;      // accumulator columns per coordinate
  static constexpr int DG = 256 / PPC;
  static constexpr int BN = ((DG * PPC + 15) / 16) * 16;
  // the adjoint's d raw: OPC bf16 columns per coordinate (FlowGeom::spl_opc),
  // one [128 rows][OPC] staging box per coordinate of the group
  static constexpr int OPC = (P + 7) / 8 * 8;
  static_assert(OPC / 8 == 1 || OPC / 8 == 2 || OPC / 8 == 4 || (OPC / 8) % 2 == 1, "d-raw box swizzle");
  static constexpr int STG_BYTES = DG * BM * OPC * 2;
};

// The first N of the PPC accumulator columns at taddr (a multiple of 8
// columns), read with 32- and 8-column loads (tcgen05.ld .32x32b.x32 / .x8 at
// 8-aligned columns); every register is pinned after the wait so no use can
// be scheduled before the data arrive.
template <int N, int PPC>
__device__ __forceinline__ void tmem_ld_coord(uint32_t taddr, float (&v)[N]) {
  static_assert(N <= PPC, "column pitch");
  uint32_t r[PPC];
  if constexpr (PPC % 8 != 0) {
    // any other pitch: one column per load
#pragma unroll
    for (int i = 0; i < N; ++i)
      asm volatile("tcgen05.ld.sync.aligned.32x32b.x1.b32 {%0}, [%1];" : "=r"(r[i]) : "r"(taddr + (uint32_t)i));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < N; ++i) {
      asm volatile("" : "+r"(r[i]));
      v[i] = __uint_as_float(r[i]);
    }
    return;
  }
  // 32-column loads while 32 columns remain, then 8-column loads
  constexpr int N32 = PPC / 32 * 32;
#pragma unroll
  for (int i = 0; i < N32; i += 32)
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[i]), "=r"(r[i + 1]), "=r"(r[i + 2]), "=r"(r[i + 3]), "=r"(r[i + 4]), "=r"(r[i + 5]),
          "=r"(r[i + 6]), "=r"(r[i + 7]), "=r"(r[i + 8]), "=r"(r[i + 9]), "=r"(r[i + 10]), "=r"(r[i + 11]),
          "=r"(r[i + 12]), "=r"(r[i + 13]), "=r"(r[i + 14]), "=r"(r[i + 15]), "=r"(r[i + 16]), "=r"(r[i + 17]),
          "=r"(r[i + 18]), "=r"(r[i + 19]), "=r"(r[i + 20]), "=r"(r[i + 21]), "=r"(r[i + 22]), "=r"(r[i + 23]),
          "=r"(r[i + 24]), "=r"(r[i + 25]), "=r"(r[i + 26]), "=r"(r[i + 27]), "=r"(r[i + 28]), "=r"(r[i + 29]),
          "=r"(r[i + 30]), "=r"(r[i + 31])
        : "r"(taddr + (uint32_t)i));
#pragma unroll
  for (int i = N32; i < PPC; i += 8)
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=r"(r[i]), "=r"(r[i + 1]), "=r"(r[i + 2]), "=r"(r[i + 3]), "=r"(r[i + 4]), "=r"(r[i + 5]),
                   "=r"(r[i + 6]), "=r"(r[i + 7])
                 : "r"(taddr + (uint32_t)i));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < PPC; ++i) asm volatile("" : "+r"(r[i]));
#pragma unroll
  for (int i = 0; i < N; ++i) v[i] = __uint_as_float(r[i]);
}

// N consecutive accumulator columns of this thread's lane, one column per load
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

// barriers and TMEM of one CTA of the fused kernels
struct Pipe {
  uint8_t* base;
  uint64_t *full, *empty, *acc_full, *acc_empty, *mma_done;
  uint32_t* tmem_slot;
  volatile int* abort_flag;
  uint32_t tmem;
};

// Ring of the one-CTA spline kernels: STAGES stages of CH consecutive 64-wide
// K chunks, A's chunks ([128 rows][128 B] each) then the weights' chunks
// ([BN rows][128 B] each), 128-byte swizzle. With CH = 1 a stage is one 2-D
// TMA box per operand; with CH > 1 it is one 3-D box {64, rows, CH} per
// operand (the chunk index as the third coordinate, stride 128 bytes), so a
// stage costs the producer two TMA operations whatever its depth in K.
template <int BN, int STAGES, int CH>
struct SplSmem {
  static constexpr int A_CH = BM * BK * 2;
  static constexpr int B_CH = BN * BK * 2;
  static constexpr int A_BYTES = CH * A_CH;
  static constexpr int B_BYTES = CH * B_CH;
  static constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
  static constexpr int TOTAL = STAGES * STAGE_BYTES + 1024 /*align slack*/ + 256 /*barriers*/;
  static_assert(A_CH % 1024 == 0 && B_CH % 1024 == 0, "swizzle atoms");
};

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1,
                                            int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], [%2];"
      ::"r"(smem_u32(dst)), "l"((uint64_t)map), "r"(smem_u32(bar)), "r"(c0), "r"(c1), "r"(c2)
      : "memory");
}

template <int BN, int STAGES, int CH>
__device__ __forceinline__ Pipe pipe_setup(uint8_t* base, int warp) {
  using S = SplSmem<BN, STAGES, CH>;
  Pipe p;
  p.base = base;
  p.full = (uint64_t*)(base + STAGES * S::STAGE_BYTES);
  p.empty = p.full + STAGES;
  p.acc_full = p.empty + STAGES;
  p.acc_empty = p.acc_full + 2;
  p.mma_done = p.acc_empty + 2;
  p.tmem_slot = (uint32_t*)(p.mma_done + 1);
  p.abort_flag = (volatile int*)(p.tmem_slot + 1);
  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&p.full[s], 1);
      mbar_init(&p.empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&p.acc_full[b], 1);
      mbar_init(&p.acc_empty[b], kSplEpiWarps);
    }
    mbar_init(p.mma_done, 1);
    *p.abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(p.tmem_slot)),
                 "r"(512));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  p.tmem = *p.tmem_slot;
  return p;
}

// warp 0, one lane: A and B K-chunks of every tile of this CTA into the ring
// (nk = stages per tile: K chunks / CH)
template <int BN, int STAGES, int CH>
__device__ __forceinline__ void producer(const Pipe& p, const CUtensorMap* tmA, const CUtensorMap* tmB, int tiles,
                                         int n_groups, int nk) {
  using S = SplSmem<BN, STAGES, CH>;
  uint32_t it = 0;
  for (int t = blockIdx.x; t < tiles && !*p.abort_flag; t += gridDim.x) {
    const int m0 = (t / n_groups) * BM, n0 = (t % n_groups) * BN;
    for (int k = 0; k < nk; ++k, ++it) {
      const int s = it % STAGES;
      const uint32_t ph = (it / STAGES) & 1u;
      if (it >= (uint32_t)STAGES && !mbar_wait(&p.empty[s], ph ^ 1u)) {
        *p.abort_flag = 1;
        break;
      }
      if (*p.abort_flag) break;
      uint8_t* sa = p.base + s * S::STAGE_BYTES;
      uint8_t* sb = sa + S::A_BYTES;
      mbar_expect_tx(&p.full[s], S::STAGE_BYTES);
      if constexpr (CH == 1) {
        tma_load_2d(sa, tmA, &p.full[s], k * BK, m0);
        tma_load_2d(sb, tmB, &p.full[s], k * BK, n0);
      } else {
        tma_load_3d(sa, tmA, &p.full[s], 0, m0, k * CH);
        tma_load_3d(sb, tmB, &p.full[s], 0, n0, k * CH);
      }
    }
  }
  if (*p.abort_flag) {
    // let the copies still in flight land before the CTA exits (bounded)
    for (uint32_t j = it > (uint32_t)STAGES ? it - STAGES : 0; j < it; ++j)
      mbar_wait(&p.full[j % STAGES], (j / STAGES) & 1u);
  }
}

// warp 1, one lane: the MMAs of every tile into accumulator (local & 1), in
// K order whatever CH is (the same sums, bit for bit)
template <int BN, int STAGES, int CH>
__device__ __forceinline__ void mma_issuer(const Pipe& p, int tiles, int nk) {
  using S = SplSmem<BN, STAGES, CH>;
  const uint32_t idesc = idesc_bf16_f32(BN);
  uint32_t it = 0;
  int local = 0;
  for (int t = blockIdx.x; t < tiles && !*p.abort_flag; t += gridDim.x, ++local) {
    const int b = local & 1, use = local >> 1;
    if (use > 0 && !mbar_wait(&p.acc_empty[b], (uint32_t)(use - 1) & 1u)) {
      *p.abort_flag = 1;
      break;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t dcol = p.tmem + (uint32_t)(b * 256);
    bool stop = false;
    for (int k = 0; k < nk; ++k, ++it) {
      const int s = it % STAGES;
      const uint32_t ph = (it / STAGES) & 1u;
      if (!mbar_wait(&p.full[s], ph) || *p.abort_flag) {
        *p.abort_flag = 1;
        stop = true;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint8_t* sa = p.base + s * S::STAGE_BYTES;
      const uint8_t* sb = sa + S::A_BYTES;
#pragma unroll
      for (int c = 0; c < CH; ++c) {
        const uint64_t da = smem_desc_sw128(sa + c * S::A_CH), db = smem_desc_sw128(sb + c * S::B_CH);
#pragma unroll
        for (int kk = 0; kk < BK / 16; ++kk)
          mma_bf16(dcol, da + (uint64_t)(kk * 2), db + (uint64_t)(kk * 2), idesc,
                   (k > 0 || c > 0 || kk > 0) ? 1u : 0u);
      }
      mma_commit(&p.empty[s]);
    }
    if (stop) break;
    mma_commit(&p.acc_full[b]);
  }
  // fires once every MMA issued so far has finished (also after an abort)
  mma_commit(p.mma_done);
}

__device__ __forceinline__ void pipe_teardown(const Pipe& p, int warp, int lane, int* err) {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    if (lane == 0) mbar_wait(p.mma_done, 0);
    __syncwarp();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(p.tmem), "r"(512));
  }
  if (threadIdx.x == 0 && *p.abort_flag) atomicExch(err, 1);
}

// this warp's TMEM lanes of accumulator b are read: hand them back to the MMA warp
__device__ __forceinline__ void release_acc(const Pipe& p, int b, int lane) {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncwarp();
  if (lane == 0) mbar_arrive(&p.acc_empty[b]);
}

// named barrier over the epilogue warps only (id 0 is __syncthreads)
__device__ __forceinline__ void epi_sync(int id) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(kSplEpiThreads) : "memory");
}

// OR of v over the epilogue warps (barrier 3 with a predicate reduction), so
// that every epilogue warp takes the same branch before a named barrier
__device__ __forceinline__ bool epi_any(bool v) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.u32 q, %1, 0;\n barrier.red.or.pred p, 3, %2, q;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(r)
      : "r"((uint32_t)v), "r"(kSplEpiThreads)
      : "memory");
  return r != 0;
}

// bias rows in shared memory: P floats per transformed coordinate, padded to
// a multiple of 4 so each row is read as float4
template <int K>
struct BiasRows {
  static constexpr int PP = (3 * K + 1 + 3) / 4 * 4;
};

// x tiles staged through shared memory (x_tma): the group's column span of
// a 128-row tile -- 2 DG floats per row, the transformed coordinates and the
// conditioning ones between them -- is one TMA box of the fp32 tensor map
// tmX over x [M, d]. The first epilogue warp's lane 0 loads the next tile's
// box while the current tile is computed (two buffers) and, after the
// epilogue warps have written y into the buffer, stores the box back. Every
// tile owns its rows' column span alone, so the write-back (which also
// rewrites the untouched conditioning columns with their own values) races
// with nothing. Without x_tma (row stride not a multiple of 16 bytes) each
// thread reads and writes its coordinates of x directly.
//
// Next-layer fold (fold_th != nullptr, x boxes only, even n_dim): the box
// leaves with the next coupling layer's ScalarAffine applied to every
// coordinate (its scale and shift at fold_th[0], fold_th[1], the pass's
// direction), and the next layer's bf16 conditioning block -- the affined
// transformed coordinates of this layer, conditioning index t -- is written
// to cond16 [M, ldc16]; that layer then needs no separate affine launch.
template <int KB, bool INV, int STAGES, int CH>
__global__ void __launch_bounds__(kSplThreads, 1)
    k_tc_spline(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                const __grid_constant__ CUtensorMap tmX, int x_tma, int M, int n_groups, int nt, int K,
                const float* __restrict__ bias, int bias_smem, float* __restrict__ xa, int d, int tpar,
                float* __restrict__ ldp, SplineCfg cfg, const float* __restrict__ fold_th,
                uint16_t* __restrict__ cond16, int ldc16, int* err) {
  using T = SplineTile<KB>;
  constexpr int P = T::P, DG = T::DG, BN = T::BN, E = kSplineEpiPerQuarter, PP = BiasRows<KB>::PP;
  constexpr int XS = 2 * DG;   // floats per row of an x box
  using S = SplSmem<BN, STAGES, CH>;
  if (tc_skip(err)) return;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* base = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  float* sbias = (float*)(base + STAGES * S::STAGE_BYTES + 256);   // after the ring and its barriers
  uint64_t* xfull = (uint64_t*)(base + STAGES * S::STAGE_BYTES + 192);   // [2], in the barrier block
  float* xbuf = (float*)((((uintptr_t)(sbias + (bias_smem ? nt * PP : 0))) + 127) & ~(uintptr_t)127);
  float* lred = xbuf + 2 * BM * XS;   // [2][E][BM] log-det partials of a tile (x boxes only)
  if (bias_smem) {
    for (int i = threadIdx.x; i < nt * PP; i += blockDim.x) {
      const int t = i / PP, pp = i - t * PP;
      sbias[i] = pp < P ? __ldg(bias + t * P + pp) : 0.f;
    }   // visible after pipe_setup's __syncthreads
  }
  if (threadIdx.x == 0) {
    mbar_init(&xfull[0], 1);
    mbar_init(&xfull[1], 1);   // pipe_setup's fence and barrier publish these
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nk = (K + BK * CH - 1) / (BK * CH);   // stages per tile (K a multiple of BK * CH when CH > 1)
  const int tiles = (M + BM - 1) / BM * n_groups;
  const Pipe p = pipe_setup<BN, STAGES, CH>(base, warp);

  if (warp == 0) {
    if (lane == 0) producer<BN, STAGES, CH>(p, &tmA, &tmB, tiles, n_groups, nk);
  } else if (warp == 1) {
    if (lane == 0) mma_issuer<BN, STAGES, CH>(p, tiles, nk);
  } else {
    const int q = warp & 3;          // TMEM lane quarter
    const int h = (warp - 2) >> 2;   // coordinates h, h + E, ... of the group
    const int row = q * 32 + lane;
    const bool xt = x_tma != 0;
    const bool elect = warp == 2 && lane == 0;   // issues the x boxes' copies
    // the next layer's affine (common.py:229, 238), as its own launch would apply it
    const bool fold = fold_th != nullptr;
    const float fs = fold ? fold_th[0] : 0.f, ft = fold ? fold_th[1] : 0.f;
    const float fes = expf(INV ? -fs : fs);
    auto next_affine = [&](float v) { return scalar_affine(v, fes, ft, INV ? 1 : 0); };
    constexpr uint32_t kXBytes = BM * XS * 4;
    int issued = 0;   // x boxes loaded so far (by the elected lane)
    if (xt && elect && (int)blockIdx.x < tiles) {
      const int t0 = blockIdx.x;
      mbar_expect_tx(&xfull[0], kXBytes);
      tma_load_2d(xbuf, &tmX, &xfull[0], 2 * (t0 % n_groups) * DG, (t0 / n_groups) * BM);
      issued = 1;
    }
    int local = 0;
    for (int t = blockIdx.x; t < tiles; t += gridDim.x, ++local) {
      const int b = local & 1, use = local >> 1;
      const int m0 = (t / n_groups) * BM, g = t % n_groups;
      const int gm = m0 + row;
      float* xb = xbuf + b * (BM * XS);
      if (xt && elect) {
        // the next tile's box goes into the other buffer once the previous
        // tile's store has finished reading it
        bulk_wait_read_0();
        const int tn = t + (int)gridDim.x;
        if (tn < tiles) {
          mbar_expect_tx(&xfull[b ^ 1], kXBytes);
          tma_load_2d(xbuf + (b ^ 1) * (BM * XS), &tmX, &xfull[b ^ 1], 2 * (tn % n_groups) * DG,
                      (tn / n_groups) * BM);
          ++issued;
        }
      }
      // every epilogue warp leaves the loop at the same tile (named barriers follow)
      bool bad = *p.abort_flag || !mbar_wait(&p.acc_full[b], (uint32_t)use & 1u);
      if (xt && !bad) bad = !mbar_wait(&xfull[b], (uint32_t)use & 1u);
      if (epi_any(bad)) {
        *p.abort_flag = 1;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t tb = p.tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * 256);
      float ldsum = 0.f;
#pragma unroll 1
      for (int u = h; u < DG; u += E) {
        const int tcoord = g * DG + u;
        if (tcoord >= nt) break;
        float raw[P];
        tmem_ld_coord<P, T::PPC>(tb + (uint32_t)(u * T::PPC), raw);   // warp-collective: every lane loads
        if (gm < M) {
          float* xp = xt ? xb + row * XS + 2 * u + tpar : xa + (int64_t)gm * d + 2 * tcoord + tpar;
          const float xv = *xp;
          if (bias_smem) {
            const float4* bb = reinterpret_cast<const float4*>(sbias + tcoord * PP);
            float bl[PP];
#pragma unroll
            for (int i = 0; i < PP / 4; ++i) {
              const float4 bv = bb[i];
              bl[4 * i] = bv.x;
              bl[4 * i + 1] = bv.y;
              bl[4 * i + 2] = bv.z;
              bl[4 * i + 3] = bv.w;
            }
            add_f2<P>(raw, bl);
          } else {
            const float* bb = bias + (int64_t)tcoord * P;
#pragma unroll
            for (int i = 0; i < P; ++i) raw[i] += __ldg(bb + i);
          }
          float y, l;
          rqs_apply_fast<KB, INV>(raw, xv, cfg, y, l);
          if (fold) {
            // this coordinate and its conditioning partner in the box (the
            // partner is conditioning here, transformed by the next layer)
            y = next_affine(y);
            float* cp = xb + row * XS + 2 * u + (1 - tpar);
            *cp = next_affine(*cp);
          }
          *xp = y;
          ldsum += l;
        }
      }
      // log-det partials: with the x boxes the quarter's E warps add theirs
      // in shared memory (two tile-parity buffers: a warp may start the next
      // tile while warp 0 of its quarter still reads this one) and one
      // partial per group and row is written; otherwise one per warp.
      // Partial-major: a warp writes 128 contiguous bytes.
      if (xt)
        lred[(b * E + h) * BM + row] = ldsum;
      else if (gm < M)
        ldp[(int64_t)(E * g + h) * M + gm] = ldsum;
      release_acc(p, b, lane);
      if (xt) {
        // y is in the buffer: make the writes visible to the copy engine, then
        // one lane stores the box (rows past M are clipped by the store)
        fence_proxy_async_smem();
        epi_sync(1);
        if (elect) {
          tma_store_2d_f32(&tmX, smem_u32(xb), 2 * g * DG, m0);
          bulk_commit();
        }
        if (h == 0 && gm < M) {
          float sl = 0.f;
#pragma unroll
          for (int k = 0; k < E; ++k) sl += lred[(b * E + k) * BM + row];
          ldp[(int64_t)g * M + gm] = sl;
          if (fold) {
            // the row's next-layer conditioning values, bf16, two per 4-byte
            // store (DG is even; the group's last coordinate may be alone)
            const int t0 = g * DG, tn = nt - t0 < DG ? nt - t0 : DG;
            const float* yr = xb + row * XS + tpar;
            uint16_t* cr = cond16 + (int64_t)gm * ldc16 + t0;
            int u = 0;
            for (; u + 1 < tn; u += 2)
              *reinterpret_cast<uint32_t*>(cr + u) =
                  (uint32_t)f32_to_bf16_rn(yr[2 * u]) | ((uint32_t)f32_to_bf16_rn(yr[2 * u + 2]) << 16);
            if (u < tn) cr[u] = f32_to_bf16_rn(yr[2 * u]);
          }
        }
      }
    }
    if (xt && elect) {
      bulk_wait_all();   // the stores have completed before the CTA exits
      // boxes loaded for tiles the loop did not finish (after an abort) land first (bounded)
      for (int k = local; k < issued; ++k) mbar_wait(&xfull[k & 1], (uint32_t)(k >> 1) & 1u);
    }
  }
  pipe_teardown(p, warp, lane, err);
}

// Arguments of the adjoint epilogue.
struct SplineBwdArgs {
  const float* bias;   // the last Linear's bias, [nt * P]
  const float* xa;     // spline inputs (the ScalarAffine output), [M, d]
  const float* gy;     // dL/d(layer output), [M, d]
  float gld;           // dL/d(log-determinant), the same for every row
  float* gxa;          // dL/d(spline input), [M, d]; conditioning coordinates copied from gy
  float* bpart;        // [m_tiles * kSplineBwdRowParts, nt*P] column sums of each 128-row tile, by row part
  int d, nt, tpar, cpar;
};

// Shared-memory position of 16-byte chunk j of row r in a d-raw staging box
// (OPC bf16 per row): the chunk order the box's TMA swizzle expects, so the
// 32 rows of a warp land in distinct banks -- none for an odd number of
// chunks per row, 32-byte swizzle for two, 64-byte swizzle for four.
template <int OCH>
__device__ __forceinline__ int draw_chunk(int r, int j) {
  if constexpr (OCH == 2) return j ^ ((r >> 2) & 1);
  if constexpr (OCH == 4) return j ^ ((r >> 1) & 3);
  return j;
}

// With x_tma the group's column span of x and of dL/dy for a 128-row tile
// arrive as two TMA boxes (loaded one tile ahead, two buffers each), the
// adjoint is written into the dL/dy box in place -- its conditioning columns
// keep dL/dy, which is their dL/dx -- and the box is stored to gxa. Each tile
// owns its rows' column span, as in the forward kernel. d raw of coordinate t
// is staged as a [128 rows][OPC] box (its P values, zeros up to OPC) and
// stored by TMA to columns [t * OPC, (t + 1) * OPC) of graw (tmR).
template <int KB, int STAGES>
__global__ void __launch_bounds__(kSplThreads, 1)
    k_tc_spline_bwd(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                    const __grid_constant__ CUtensorMap tmX, const __grid_constant__ CUtensorMap tmGy,
                    const __grid_constant__ CUtensorMap tmGx, const __grid_constant__ CUtensorMap tmR, int x_tma,
                    int M, int n_groups, int K, const SplineBwdArgs a, SplineCfg cfg, int* err) {
  using T = SplineTile<KB>;
  constexpr int P = T::P, DG = T::DG, BN = T::BN, E = kSplineEpiPerQuarter;
  constexpr int OPC = T::OPC, OCH = OPC / 8, OBOX = BM * OPC * 2;
  constexpr int CP = DG * OPC / 2;                 // column pairs of a group's staged boxes
  constexpr int RP = kSplineBwdRowParts;
  constexpr int RROWS = (BM + RP - 1) / RP;        // rows per column-sum part
  static_assert(RP * CP <= kSplEpiThreads, "one thread per column pair and row part");
  constexpr int XS = 2 * DG;   // floats per row of a box
  using S = SplSmem<BN, STAGES, 1>;
  if (tc_skip(err)) return;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* base = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  // staging boxes 1024 bytes after the ring (the barrier block between), then the x / dL/dy boxes
  uint8_t* stg = base + STAGES * S::STAGE_BYTES + 1024;
  uint64_t* xfull = (uint64_t*)(base + STAGES * S::STAGE_BYTES + 192);   // [2], in the barrier block
  float* boxes = (float*)(stg + DG * OBOX);                                 // [2][x | dL/dy]
  if (threadIdx.x == 0) {
    mbar_init(&xfull[0], 1);
    mbar_init(&xfull[1], 1);   // pipe_setup's fence and barrier publish these
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nk = (K + BK - 1) / BK;
  const int tiles = (M + BM - 1) / BM * n_groups;
  const int ntP = a.nt * P;
  const Pipe p = pipe_setup<BN, STAGES, 1>(base, warp);

  if (warp == 0) {
    if (lane == 0) producer<BN, STAGES, 1>(p, &tmA, &tmB, tiles, n_groups, nk);
  } else if (warp == 1) {
    if (lane == 0) mma_issuer<BN, STAGES, 1>(p, tiles, nk);
  } else {
    const int q = warp & 3;
    const int h = (warp - 2) >> 2;
    const int row = q * 32 + lane;
    const int et = threadIdx.x - 64;   // 0 .. kSplEpiThreads-1
    const bool xt = x_tma != 0;
    const bool elect = warp == 2 && lane == 0;   // issues the boxes' copies
    constexpr uint32_t kBox = BM * XS;           // floats per box
    auto load_boxes = [&](int tt, int buf) {
      float* xb = boxes + (2 * buf) * kBox;
      mbar_expect_tx(&xfull[buf], 2 * kBox * 4);
      tma_load_2d(xb, &tmX, &xfull[buf], 2 * (tt % n_groups) * DG, (tt / n_groups) * BM);
      tma_load_2d(xb + kBox, &tmGy, &xfull[buf], 2 * (tt % n_groups) * DG, (tt / n_groups) * BM);
    };
    int issued = 0;
    if (xt && elect && (int)blockIdx.x < tiles) {
      load_boxes(blockIdx.x, 0);
      issued = 1;
    }
    int local = 0;
    for (int t = blockIdx.x; t < tiles; t += gridDim.x, ++local) {
      const int b = local & 1, use = local >> 1;
      const int mt = t / n_groups, g = t % n_groups;
      const int m0 = mt * BM;
      const int gm = m0 + row;
      const bool row_ok = gm < M;
      float* xb = boxes + (2 * b) * kBox;
      float* gb = xb + kBox;
      if (xt && elect) {
        // the next tile's boxes go into the other buffers (every earlier
        // store finished reading shared memory at the end of the last tile)
        const int tn = t + (int)gridDim.x;
        if (tn < tiles) {
          load_boxes(tn, b ^ 1);
          ++issued;
        }
      }
      // the tile loop has named barriers: all epilogue warps leave it together
      bool bad = *p.abort_flag || !mbar_wait(&p.acc_full[b], (uint32_t)use & 1u);
      if (xt && !bad) bad = !mbar_wait(&xfull[b], (uint32_t)use & 1u);
      if (epi_any(bad)) {
        *p.abort_flag = 1;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t tb = p.tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * 256);
      const int nu = (a.nt - g * DG) < DG ? (a.nt - g * DG) : DG;   // coordinates in this group
#pragma unroll 1
      for (int u = h; u < nu; u += E) {
        const int tcoord = g * DG + u;
        float raw[P];
        tmem_ld_coord<P, T::PPC>(tb + (uint32_t)(u * T::PPC), raw);
        uint16_t ov[OPC];   // this row's d raw of coordinate u, zeros past P
#pragma unroll
        for (int i = 0; i < OPC; ++i) ov[i] = 0;
        if (row_ok) {
          const float* bb = a.bias + (int64_t)tcoord * P;
#pragma unroll
          for (int i = 0; i < P; ++i) raw[i] += __ldg(bb + i);
          if (xt) {
            const int jb = row * XS + 2 * u + a.tpar;
            gb[jb] = rqs_fwd_adjoint_fast<KB>(raw, xb[jb], gb[jb], a.gld, cfg, ov);
          } else {
            const int64_t j = (int64_t)gm * a.d + 2 * tcoord + a.tpar;
            a.gxa[j] = rqs_fwd_adjoint_fast<KB>(raw, a.xa[j], a.gy[j], a.gld, cfg, ov);
          }
        }
        // the row's OCH 16-byte chunks into the coordinate's staging box
        const uint32_t rb = smem_u32(stg + u * OBOX + row * (OPC * 2));
#pragma unroll
        for (int j = 0; j < OCH; ++j) {
          uint32_t w4[4];
#pragma unroll
          for (int k = 0; k < 4; ++k) w4[k] = (uint32_t)ov[8 * j + 2 * k] | ((uint32_t)ov[8 * j + 2 * k + 1] << 16);
          st_shared_v4(rb + (uint32_t)(draw_chunk<OCH>(row, j) * 16), w4[0], w4[1], w4[2], w4[3]);
        }
      }
      release_acc(p, b, lane);
      if (!xt && g == 0 && row_ok) {
        const int ncond = a.d - a.nt;
        for (int k = h; k < ncond; k += E) {
          const int64_t j = (int64_t)gm * a.d + 2 * k + a.cpar;
          a.gxa[j] = a.gy[j];
        }
      }
      // the staged boxes' generic writes, before the copy engine reads them
      fence_proxy_async_smem();
      epi_sync(1);
      if (elect) {
        if (xt) tma_store_2d_f32(&tmGx, smem_u32(gb), 2 * g * DG, m0);
        for (int u = 0; u < nu; ++u) tma_store_2d(&tmR, smem_u32(stg + u * OBOX), (g * DG + u) * OPC, m0);
        bulk_commit();
      }
      // column sums of d raw over the tile's rows (rows >= M were staged as
      // zeros), while the stores read the same boxes: thread e takes column
      // pair cp = e % CP of the group's boxes over row part e / CP, in row order
      if (et < RP * CP) {
        const int cp = et % CP, part = et / CP;
        const int u = cp / (OPC / 2), p2 = cp - u * (OPC / 2);
        if (u < nu && 2 * p2 < P) {
          const uint8_t* box = stg + u * OBOX;
          const int j = (2 * p2) >> 3, wofs = ((2 * p2) & 7) * 2;
          float s0 = 0.f, s1 = 0.f;
          const int r1 = (part + 1) * RROWS < BM ? (part + 1) * RROWS : BM;
#pragma unroll 4
          for (int r = part * RROWS; r < r1; ++r) {
            const uint32_t v =
                *reinterpret_cast<const uint32_t*>(box + r * (OPC * 2) + draw_chunk<OCH>(r, j) * 16 + wofs);
            s0 += __uint_as_float(v << 16);
            s1 += __uint_as_float(v & 0xffff0000u);
          }
          float* dst = a.bpart + (int64_t)(mt * RP + part) * ntP + (int64_t)(g * DG + u) * P + 2 * p2;
          dst[0] = s0;
          if (2 * p2 + 1 < P) dst[1] = s1;
        }
      }
      // the boxes are free again once the stores have read them
      if (elect) bulk_wait_read_0();
      epi_sync(2);
    }
    if (elect) {
      bulk_wait_all();   // the stores have completed before the CTA exits
      // boxes loaded for tiles the loop did not finish (after an abort) land first (bounded)
      if (xt)
        for (int k = local; k < issued; ++k) mbar_wait(&xfull[k & 1], (uint32_t)(k >> 1) & 1u);
    }
  }
  pipe_teardown(p, warp, lane, err);
}

// ---------------------------------------------------------------- CTA pairs
// k_tc_spline2: the same fused last Linear + spline, with (256-row, group)
// tiles computed by a CTA pair (cluster of 2, tcgen05 cta_group::2). Each
// CTA loads its 128 rows of A and half (BN / 2 rows) of the group's weights;
// the even CTA issues the M = 256 MMAs for both; each CTA runs the epilogue
// of its own 128 rows from its own TMEM. Per CTA and tile the operand traffic
// from L2 is 128 x K (A) + BN / 2 x K (B) instead of 128 x K + BN x K.
//
// Barriers: the ring's `full` barriers of the even CTA count both CTAs'
// copies (its producer arms them with both halves' bytes; the odd CTA's
// copies signal them across the pair); `empty`, `acc_full` and `mma_done`
// exist in both CTAs and are completed by the pair's commits (multicast);
// `acc_empty` of the even CTA counts the epilogue warps of both CTAs.
// Every wait is bounded; the pair agrees on the fail-fast decision first.

template <int BH, int STAGES>
struct PairSmem {
  static constexpr int A_BYTES = BM * BK * 2;
  static constexpr int B_BYTES = BH * BK * 2;
  static constexpr int STAGE_BYTES = ((A_BYTES + B_BYTES + 1023) / 1024) * 1024;
  static constexpr int RING = STAGES * STAGE_BYTES;
};

template <int BH, int STAGES>
__device__ __forceinline__ Pipe pipe_setup_pair(uint8_t* base, int warp, uint32_t rank) {
  using S = PairSmem<BH, STAGES>;
  Pipe p;
  p.base = base;
  p.full = (uint64_t*)(base + S::RING);
  p.empty = p.full + STAGES;
  p.acc_full = p.empty + STAGES;
  p.acc_empty = p.acc_full + 2;
  p.mma_done = p.acc_empty + 2;
  p.tmem_slot = (uint32_t*)(p.mma_done + 1);
  p.abort_flag = (volatile int*)(p.tmem_slot + 1);
  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&p.full[s], 1);
      mbar_init(&p.empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&p.acc_full[b], 1);
      mbar_init(&p.acc_empty[b], 2 * kSplEpiWarps);
    }
    mbar_init(p.mma_done, 1);
    *p.abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(p.tmem_slot)),
                 "r"(512));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  // both CTAs' barriers are initialised before either side signals the other's
  cluster_sync_all();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  p.tmem = *p.tmem_slot;
  (void)rank;
  return p;
}

// warp 0, one lane, in both CTAs: this CTA's A rows and B half of every tile
template <int BH, int STAGES>
__device__ __forceinline__ void producer_pair(const Pipe& p, const CUtensorMap* tmA, const CUtensorMap* tmB,
                                              int tiles, int n_groups, int nk, uint32_t rank) {
  using S = PairSmem<BH, STAGES>;
  const int n_pairs = gridDim.x / 2, pair = blockIdx.x / 2;
  uint32_t it = 0;
  for (int t = pair; t < tiles && !*p.abort_flag; t += n_pairs) {
    const int m0 = (t / n_groups) * (2 * BM) + (int)rank * BM;
    const int n0 = (t % n_groups) * (2 * BH) + (int)rank * BH;
    for (int k = 0; k < nk; ++k, ++it) {
      const int s = it % STAGES;
      const uint32_t ph = (it / STAGES) & 1u;
      if (it >= (uint32_t)STAGES && !mbar_wait(&p.empty[s], ph ^ 1u)) {
        *p.abort_flag = 1;
        break;
      }
      if (*p.abort_flag) break;
      uint8_t* sa = p.base + s * S::STAGE_BYTES;
      uint8_t* sb = sa + S::A_BYTES;
      const uint32_t full_cl = mapa_shared(smem_u32(&p.full[s]), 0);
      if (rank == 0) mbar_expect_tx(&p.full[s], 2 * (S::A_BYTES + S::B_BYTES));
      tma_load_2d_pair(sa, tmA, full_cl, k * BK, m0);
      tma_load_2d_pair(sb, tmB, full_cl, k * BK, n0);
    }
  }
  if (*p.abort_flag) {
    // this CTA's copies still in flight must land before it exits; their
    // completion is counted on the even CTA's barriers, so wait on the
    // stages' release by the MMA side instead (bounded)
    for (uint32_t j = it > (uint32_t)STAGES ? it - STAGES : 0; j < it; ++j)
      mbar_wait(&p.empty[j % STAGES], (j / STAGES) & 1u);
  }
}

// warp 1, one lane, even CTA only: the pair's MMAs of every tile
template <int BN, int BH, int STAGES>
__device__ __forceinline__ void mma_issuer_pair(const Pipe& p, int tiles, int nk) {
  using S = PairSmem<BH, STAGES>;
  const uint32_t idesc = idesc_bf16_f32_pair(BN);
  const int n_pairs = gridDim.x / 2, pair = blockIdx.x / 2;
  uint32_t it = 0;
  int local = 0;
  for (int t = pair; t < tiles && !*p.abort_flag; t += n_pairs, ++local) {
    const int b = local & 1, use = local >> 1;
    if (use > 0 && !mbar_wait_cl(&p.acc_empty[b], (uint32_t)(use - 1) & 1u)) {
      *p.abort_flag = 1;
      break;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t dcol = p.tmem + (uint32_t)(b * 256);
    bool stop = false;
    for (int k = 0; k < nk; ++k, ++it) {
      const int s = it % STAGES;
      const uint32_t ph = (it / STAGES) & 1u;
      if (!mbar_wait(&p.full[s], ph) || *p.abort_flag) {
        *p.abort_flag = 1;
        stop = true;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint8_t* sa = p.base + s * S::STAGE_BYTES;
      const uint8_t* sb = sa + S::A_BYTES;
      const uint64_t da = smem_desc_sw128(sa), db = smem_desc_sw128(sb);
#pragma unroll
      for (int kk = 0; kk < BK / 16; ++kk)
        mma_bf16_pair(dcol, da + (uint64_t)(kk * 2), db + (uint64_t)(kk * 2), idesc, (k > 0 || kk > 0) ? 1u : 0u);
      mma_commit_pair(&p.empty[s]);
    }
    if (stop) break;
    mma_commit_pair(&p.acc_full[b]);
  }
  // fires in both CTAs once every MMA issued so far has finished
  mma_commit_pair(p.mma_done);
}

__device__ __forceinline__ void pipe_teardown_pair(const Pipe& p, int warp, int lane, uint32_t rank, int* err) {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    // the even CTA's MMAs read both CTAs' shared memory and write both TMEMs
    if (lane == 0) mbar_wait_cl(p.mma_done, 0);
    __syncwarp();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(p.tmem), "r"(512));
  }
  if (threadIdx.x == 0 && *p.abort_flag) atomicExch(err, 1);
  // neither CTA leaves while the other may still signal its barriers
  cluster_sync_all();
  (void)rank;
}

template <int KB, bool INV, int STAGES>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(kSplThreads, 1)
    k_tc_spline2(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, int M,
                 int n_groups, int nt, int K, const float* __restrict__ bias, int bias_smem, float* __restrict__ xa,
                 int d, int tpar, float* __restrict__ ldp, SplineCfg cfg, int* err) {
  using T = SplineTile<KB>;
  constexpr int P = T::P, DG = T::DG, BN = T::BN, BH = BN / 2, E = kSplineEpiPerQuarter, PP = BiasRows<KB>::PP;
  static_assert(BN % 32 == 0, "a CTA pair splits the group's weight rows in two multiples of 16");
  using S = PairSmem<BH, STAGES>;
  if (tc_skip_pair(err)) return;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* base = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  float* sbias = (float*)(base + S::RING + 256 + S::B_BYTES);   // after the ring, its barriers and the slack
  if (bias_smem) {
    for (int i = threadIdx.x; i < nt * PP; i += blockDim.x) {
      const int t = i / PP, pp = i - t * PP;
      sbias[i] = pp < P ? __ldg(bias + t * P + pp) : 0.f;
    }   // visible after the set-up's barriers
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t rank = cluster_ctarank();
  const int nk = (K + BK - 1) / BK;
  const int tiles = (M + 2 * BM - 1) / (2 * BM) * n_groups;
  const Pipe p = pipe_setup_pair<BH, STAGES>(base, warp, rank);
  const uint32_t acc_empty_cl0 = mapa_shared(smem_u32(&p.acc_empty[0]), 0);
  const uint32_t acc_empty_cl1 = mapa_shared(smem_u32(&p.acc_empty[1]), 0);

  if (warp == 0) {
    if (lane == 0) producer_pair<BH, STAGES>(p, &tmA, &tmB, tiles, n_groups, nk, rank);
  } else if (warp == 1) {
    if (lane == 0 && rank == 0) mma_issuer_pair<BN, BH, STAGES>(p, tiles, nk);
  } else {
    const int q = warp & 3;          // TMEM lane quarter
    const int h = (warp - 2) >> 2;   // coordinates h, h + E, ... of the group
    const int row = q * 32 + lane;
    const int n_pairs = gridDim.x / 2, pair = blockIdx.x / 2;
    int local = 0;
    for (int t = pair; t < tiles; t += n_pairs, ++local) {
      const int b = local & 1, use = local >> 1;
      const int m0 = (t / n_groups) * (2 * BM) + (int)rank * BM, g = t % n_groups;
      const int gm = m0 + row;
      if (*p.abort_flag || !mbar_wait(&p.acc_full[b], (uint32_t)use & 1u)) {
        *p.abort_flag = 1;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t tb = p.tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * 256);
      float ldsum = 0.f;
#pragma unroll 1
      for (int u = h; u < DG; u += E) {
        const int tcoord = g * DG + u;
        if (tcoord >= nt) break;
        float raw[P];
        tmem_ld_coord<P, T::PPC>(tb + (uint32_t)(u * T::PPC), raw);   // warp-collective: every lane loads
        if (gm < M) {
          float* xp = xa + (int64_t)gm * d + 2 * tcoord + tpar;
          const float xv = *xp;
          if (bias_smem) {
            const float4* bb = reinterpret_cast<const float4*>(sbias + tcoord * PP);
            float bl[PP];
#pragma unroll
            for (int i = 0; i < PP / 4; ++i) {
              const float4 bv = bb[i];
              bl[4 * i] = bv.x;
              bl[4 * i + 1] = bv.y;
              bl[4 * i + 2] = bv.z;
              bl[4 * i + 3] = bv.w;
            }
            add_f2<P>(raw, bl);
          } else {
            const float* bb = bias + (int64_t)tcoord * P;
#pragma unroll
            for (int i = 0; i < P; ++i) raw[i] += __ldg(bb + i);
          }
          float y, l;
          rqs_apply_fast<KB, INV>(raw, xv, cfg, y, l);
          *xp = y;
          ldsum += l;
        }
      }
      if (gm < M) ldp[(int64_t)(E * g + h) * M + gm] = ldsum;   // partial-major: a warp writes 128 contiguous bytes
      // this warp's TMEM lanes of accumulator b are read: tell the even CTA's MMA warp
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive_cluster(b ? acc_empty_cl1 : acc_empty_cl0);
    }
  }
  pipe_teardown_pair(p, warp, lane, rank, err);
}

}  // namespace tc

// ld[r] += sum of the row's kSplineEpiPerQuarter * n_groups partials (fixed
// order); partial j of row r is ldp[j * m + r]. With th_next (the spline
// kernel applied the next layer's ScalarAffine), that affine's log-determinant
// d * (+-s) is added after them, as the affine's own launch would have.
__global__ void k_ld_reduce(const float* __restrict__ ldp, int n_part, int64_t m, float* __restrict__ ld,
                            const float* __restrict__ th_next, int d, int inverse) {
  const float la = th_next != nullptr ? scalar_affine_logdet(th_next[0], d, inverse) : 0.f;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < m; r += (int64_t)gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int j = 0; j < n_part; ++j) s += ldp[(int64_t)j * m + r];
    float v = ld[r] + s;
    if (th_next != nullptr) v = __fadd_rn(v, la);
    ld[r] = v;
  }
}

// ld_reduce_steps' kernel: per row, step k's partials summed in order, added,
// then step k's folded affine log-det (k_ld_reduce's arithmetic, step by step)
__global__ void k_ld_steps(const float* __restrict__ ldp, const LdSteps s, int64_t m, float* __restrict__ ld, int d,
                           int inverse) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < m; r += (int64_t)gridDim.x * blockDim.x) {
    float v = ld[r];
    for (int k = 0; k < s.n; ++k) {
      const float* p = ldp + s.off[k] + r;
      float sum = 0.f;
      for (int j = 0; j < s.parts[k]; ++j) sum += p[(int64_t)j * m];
      v = v + sum;
      if (s.th_next[k] != nullptr) v = __fadd_rn(v, scalar_affine_logdet(s.th_next[k][0], d, inverse));
    }
    ld[r] = v;
  }
}

int ld_reduce_steps(cudaStream_t st, const float* ldp, const LdSteps& s, int64_t m, float* ld, int d, bool inverse) {
  FMC_CHECK_ARG(s.n >= 0 && s.n <= kLdMaxSteps, "ld_reduce_steps: %d steps", s.n);
  if (s.n == 0 || m <= 0) return FMC_OK;
  int64_t blocks = (m + 255) / 256;
  if (blocks > (int64_t)sm_count() * 8) blocks = (int64_t)sm_count() * 8;
  k_ld_steps<<<(int)(blocks < 1 ? 1 : blocks), 256, 0, st>>>(ldp, s, m, ld, d, inverse ? 1 : 0);
  FMC_LAUNCH_CHECK();
  return FMC_OK;
}

int tc_error_word(int** out);
int make_tma_map_bf16(CUtensorMap* m, const void* base, int64_t inner, int64_t outer, int64_t ld, int box_outer);
int make_tma_map_f32(CUtensorMap* m, const void* base, int64_t inner, int64_t outer, int box_inner, int box_outer);
int make_tma_map_bf16_box(CUtensorMap* m, const void* base, int64_t inner, int64_t outer, int64_t ld, int box_inner,
                          int box_outer, int swizzle);
int make_tma_map_bf16_chunks(CUtensorMap* m, const void* base, int64_t inner, int64_t outer, int64_t ld,
                             int box_outer, int ch);

int spline_groups(int K_bins, int nt, int* dg, int* bn) {
  const int P = 3 * K_bins + 1, PP = (P + 7) / 8 * 8;
  const int DG = 256 / PP;
  *dg = DG;
  *bn = ((DG * PP + 15) / 16) * 16;
  return (nt + DG - 1) / DG;
}

// CH K chunks per ring stage: 4 one-chunk stages, or 2 two-chunk stages
// (3-D operand maps; half the TMA operations per tile, measured 3-4 % faster
// on GB300 at 512 hidden units)
template <int KB, bool INV, int CH>
static int launch_spl(cudaStream_t st, const CUtensorMap& ma, const CUtensorMap& mb, int64_t M, int n_groups, int nt,
                      int K, const float* bias, float* xa, int d, int tpar, float* ldp, SplineCfg cfg, int* parts,
                      const SplineFold* fold, bool* folded) {
  constexpr int STAGES = CH == 1 ? 4 : 2;
  using T = tc::SplineTile<KB>;
  using S = tc::SplSmem<T::BN, STAGES, CH>;
  auto kern = tc::k_tc_spline<KB, INV, STAGES, CH>;
  // the ring, its barriers, (when they fit) the layer's bias rows and the two
  // x boxes (when x's row stride allows a tensor map)
  const size_t bias_bytes = (size_t)nt * tc::BiasRows<KB>::PP * sizeof(float);
  // the two x boxes and the per-tile log-det partials of the quarter's warps
  const size_t x_bytes = 128 + 2 * (size_t)tc::BM * 2 * T::DG * sizeof(float) +
                         2 * (size_t)kSplineEpiPerQuarter * tc::BM * sizeof(float);
  CUtensorMap mx;
  memset(&mx, 0, sizeof(mx));
  int x_tma = make_tma_map_f32(&mx, xa, d, M, 2 * T::DG, tc::BM) == FMC_OK ? 1 : 0;
  if (!x_tma) (void)cudaGetLastError();
  if (x_tma && S::TOTAL + x_bytes > 227 * 1024) x_tma = 0;
  const size_t base_bytes = (size_t)S::TOTAL + (x_tma ? x_bytes : 0);
  const int bias_smem = base_bytes + bias_bytes <= 227 * 1024 ? 1 : 0;
  const size_t total = base_bytes + (bias_smem ? bias_bytes : 0);
  static int attr = 0;
  if (attr < (int)total) {
    FMC_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)total));
    attr = (int)total;
  }
  int* err = nullptr;
  int rc = tc_error_word(&err);
  if (rc) return rc;
  const int64_t tiles = (M + tc::BM - 1) / tc::BM * n_groups;
  const int64_t grid = tiles < sm_count() ? tiles : sm_count();
  note_grid(INV ? FMC_KT_TC_SPLINE_INV : FMC_KT_TC_SPLINE_FWD, (int)grid, 1);
  // the next layer's affine rides on the x boxes only
  const bool fo = fold != nullptr && x_tma;
  kern<<<(unsigned)grid, tc::kSplThreads, total, st>>>(ma, mb, mx, x_tma, (int)M, n_groups, nt, K, bias, bias_smem,
                                                       xa, d, tpar, ldp, cfg, fo ? fold->th_next : nullptr,
                                                       fo ? fold->cond16 : nullptr, fo ? fold->ldc16 : 0, err);
  FMC_LAUNCH_CHECK();
  *parts = x_tma ? n_groups : kSplineEpiPerQuarter * n_groups;
  *folded = fo;
  return FMC_OK;
}

// the CTA-pair variant: a persistent grid of as many pairs as can be resident
template <int KB, bool INV>
static int launch_spl2(cudaStream_t st, const CUtensorMap& ma, const CUtensorMap& mb, int64_t M, int n_groups, int nt,
                       int K, const float* bias, float* xa, int d, int tpar, float* ldp, SplineCfg cfg) {
  constexpr int STAGES = 6;
  using T = tc::SplineTile<KB>;
  using S = tc::PairSmem<T::BN / 2, STAGES>;
  auto kern = tc::k_tc_spline2<KB, INV, STAGES>;
  // ring, alignment slack, barriers; one B half of slack after the ring keeps
  // every operand read of the last stage inside the allocation
  const size_t ring = (size_t)S::RING + 1024 /*align slack*/ + 256 /*barriers*/;
  const size_t ring_slack = ring + (size_t)S::B_BYTES;
  const size_t with_bias = ring_slack + (size_t)nt * tc::BiasRows<KB>::PP * sizeof(float);
  const int bias_smem = with_bias <= 227 * 1024 ? 1 : 0;
  const size_t total = bias_smem ? with_bias : ring_slack;
  static int attr = 0;
  if (attr < (int)total) {
    FMC_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)total));
    attr = (int)total;
  }
  static int max_pairs = 0;
  if (max_pairs == 0) {
    cudaLaunchConfig_t cfg_l = {};
    cfg_l.gridDim = dim3(2 * (unsigned)(sm_count() / 2), 1, 1);
    cfg_l.blockDim = dim3(tc::kSplThreads, 1, 1);
    cfg_l.dynamicSmemBytes = total;
    int n = 0;
    FMC_CUDA_TRY(cudaOccupancyMaxActiveClusters(&n, (void*)kern, &cfg_l));
    max_pairs = n > 0 ? n : 1;
  }
  int* err = nullptr;
  int rc = tc_error_word(&err);
  if (rc) return rc;
  const int64_t tiles = (M + 2 * tc::BM - 1) / (2 * tc::BM) * n_groups;
  const int64_t pairs = tiles < max_pairs ? tiles : max_pairs;
  note_grid(INV ? FMC_KT_TC_SPLINE_INV : FMC_KT_TC_SPLINE_FWD, (int)(2 * pairs), 2);
  kern<<<(unsigned)(2 * pairs), tc::kSplThreads, total, st>>>(ma, mb, (int)M, n_groups, nt, K, bias, bias_smem, xa, d,
                                                             tpar, ldp, cfg, err);
  FMC_LAUNCH_CHECK();
  return FMC_OK;
}

// one-CTA tiles (two-chunk stages when the maps are the 3-D chunk maps), or
// CTA pairs where the group's weight rows split into two multiples of 16 (the
// pair kernel exists only for those widths)
template <int KB, bool INV>
static int launch_spl_tiles(bool pair, bool wide, cudaStream_t st, const CUtensorMap& ma, const CUtensorMap& mb,
                            int64_t M, int n_groups, int nt, int K, const float* bias, float* xa, int d, int tpar,
                            float* ldp, SplineCfg cfg, int* parts, const SplineFold* fold, bool* folded) {
  *folded = false;
  if constexpr (tc::SplineTile<KB>::BN % 32 == 0) {
    if (pair) {
      *parts = kSplineEpiPerQuarter * n_groups;
      return launch_spl2<KB, INV>(st, ma, mb, M, n_groups, nt, K, bias, xa, d, tpar, ldp, cfg);
    }
  }
  if (wide)
    return launch_spl<KB, INV, 2>(st, ma, mb, M, n_groups, nt, K, bias, xa, d, tpar, ldp, cfg, parts, fold, folded);
  return launch_spl<KB, INV, 1>(st, ma, mb, M, n_groups, nt, K, bias, xa, d, tpar, ldp, cfg, parts, fold, folded);
}

template <int KB>
static int launch_spl_bwd(cudaStream_t st, const CUtensorMap& ma, const CUtensorMap& mb, int64_t M, int n_groups,
                          int K, const tc::SplineBwdArgs& a, uint16_t* graw, int64_t ldg, SplineCfg cfg) {
  constexpr int STAGES = 3;
  using T = tc::SplineTile<KB>;
  using S = tc::SplSmem<T::BN, STAGES, 1>;
  // ring, slack and barrier block (S::TOTAL), the rest of a 1024-byte block, the staging boxes
  constexpr int TOTAL = S::TOTAL + 768 + T::STG_BYTES;
  static_assert(TOTAL + 16 <= 227 * 1024, "fused spline adjoint: shared memory over the per-CTA limit");
  // x and dL/dy boxes (two buffers each) when the row stride allows tensor maps and they fit
  constexpr int BOXES = 128 + 4 * tc::BM * 2 * T::DG * (int)sizeof(float);
  CUtensorMap mx, mgy, mgx;
  memset(&mx, 0, sizeof(mx));
  memset(&mgy, 0, sizeof(mgy));
  memset(&mgx, 0, sizeof(mgx));
  // d raw: one box {OPC, 128} per coordinate, swizzled as the staging is
  CUtensorMap mr;
  constexpr int och = T::OPC / 8;
  const int swz = och == 2 ? 32 : och == 4 ? 64 : 0;
  int rc = make_tma_map_bf16_box(&mr, graw, ldg, M, ldg, T::OPC, tc::BM, swz);
  if (rc) return rc;
  int x_tma = TOTAL + BOXES + 16 <= 227 * 1024 && make_tma_map_f32(&mx, a.xa, a.d, M, 2 * T::DG, tc::BM) == FMC_OK &&
              make_tma_map_f32(&mgy, a.gy, a.d, M, 2 * T::DG, tc::BM) == FMC_OK &&
              make_tma_map_f32(&mgx, a.gxa, a.d, M, 2 * T::DG, tc::BM) == FMC_OK;
  const int total = TOTAL + (x_tma ? BOXES : 0);
  auto kern = tc::k_tc_spline_bwd<KB, STAGES>;
  static int attr = 0;
  if (attr < total) {
    FMC_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, total));
    attr = total;
  }
  int* err = nullptr;
  if ((rc = tc_error_word(&err))) return rc;
  const int64_t tiles = (M + tc::BM - 1) / tc::BM * n_groups;
  const int64_t grid = tiles < sm_count() ? tiles : sm_count();
  note_grid(FMC_KT_TC_SPLINE_BWD, (int)grid, 1);
  kern<<<(unsigned)grid, tc::kSplThreads, total, st>>>(ma, mb, mx, mgy, mgx, mr, x_tma, (int)M, n_groups, K, a, cfg,
                                                       err);
  FMC_LAUNCH_CHECK();
  return FMC_OK;
}

#define FMC_SPLINE_BINS(X) X(2) X(3) X(4) X(5) X(6) X(8) X(10) X(12) X(16)

// The last Linear of layer l fused with its spline: A = the last tanh
// activation (bf16 [rows_a, K]), Bg = the grouped weights, xa updated in place,
// ld[r] accumulated.
int tc_linear_spline(cudaStream_t st, const FlowGeom& g, const FmcFlow* f, int l, const uint16_t* A, int64_t M,
                     int64_t rows_a, bool inverse, float* xa, float* ld, float* ldp, const SplineFold* fold,
                     bool* folded, int* parts_out) {
  bool fo = false;
  if (folded) *folded = false;
  // the fold pairs every conditioning coordinate with a transformed one
  if (fold != nullptr) FMC_CHECK_ARG(2 * g.nt(l) == g.d && fold->th_next && fold->cond16, "spline fold: bad arguments");
  const int nt = g.nt(l);
  int dg, bn;
  const int n_groups = spline_groups(g.K, nt, &dg, &bn);
  const int Kd = g.w16_cols(l, g.nh);
  const uint16_t* Bg = f->theta_bf16 + g.w16g_off[l];
  const float* bias = f->theta + g.layer_off[l] + g.lin_b(l, g.nh);
  // CTA pairs (256-row tiles, half the weight rows per CTA) when asked for
  // and the group width splits in two multiples of 16; one-CTA tiles by
  // default (measured faster on GB300 at the sampler's shapes)
  const bool pair = f->tile_rows == 256 && bn % 32 == 0;
  // two-chunk ring stages when K splits into 128-wide stages
  const bool wide = !pair && Kd % (2 * tc::BK) == 0;
  CUtensorMap ma, mb;
  int rc;
  if (wide) {
    if ((rc = make_tma_map_bf16_chunks(&ma, A, Kd, rows_a, Kd, tc::BM, 2))) return rc;
    if ((rc = make_tma_map_bf16_chunks(&mb, Bg, Kd, (int64_t)n_groups * bn, Kd, bn, 2))) return rc;
  } else {
    if ((rc = make_tma_map_bf16(&ma, A, Kd, rows_a, Kd, tc::BM))) return rc;
    if ((rc = make_tma_map_bf16(&mb, Bg, Kd, (int64_t)n_groups * bn, Kd, pair ? bn / 2 : bn))) return rc;
  }
  int parts = kSplineEpiPerQuarter * n_groups;   // log-det partials per row the launch leaves
  {
    // useful work: the last Linear's nt * P outputs over its H_last inputs,
    // the A rows and the group weights once, x read and written, partials
    const int hl = g.H[g.nh - 1];
    const double flops = 2.0 * (double)M * nt * g.P * hl;
    const double bytes = (double)M * hl * 2 + (double)nt * g.P * hl * 2 + (double)M * nt * 8 +
                         (double)M * kSplineEpiPerQuarter * n_groups * 4;
    KernelTimer kt(inverse ? FMC_KT_TC_SPLINE_INV : FMC_KT_TC_SPLINE_FWD, st, flops, bytes);
#define SPL_CASE(k)                                                                                          \
  if (g.K == k) {                                                                                            \
    rc = inverse                                                                                             \
             ? launch_spl_tiles<k, true>(pair, wide, st, ma, mb, M, n_groups, nt, Kd, bias, xa, g.d, g.tpar(l),  \
                                         ldp, g.cfg, &parts, fold, &fo)                                            \
             : launch_spl_tiles<k, false>(pair, wide, st, ma, mb, M, n_groups, nt, Kd, bias, xa, g.d, g.tpar(l), \
                                          ldp, g.cfg, &parts, fold, &fo);                                          \
  } else
    FMC_SPLINE_BINS(SPL_CASE) {
      set_error("n_bins=%d is not instantiated for the fused spline", g.K);
      return FMC_ERR_UNSUPPORTED;
    }
#undef SPL_CASE
  }
  if (rc) return rc;
  if (folded) *folded = fo;
  if (parts_out) *parts_out = parts;
  if (ld == nullptr) return FMC_OK;   // the caller adds the partials later
  int64_t blocks = (M + 255) / 256;
  if (blocks > (int64_t)sm_count() * 8) blocks = (int64_t)sm_count() * 8;
  k_ld_reduce<<<(int)(blocks < 1 ? 1 : blocks), 256, 0, st>>>(ldp, parts, M, ld, fo ? fold->th_next : nullptr, g.d,
                                                               inverse ? 1 : 0);
  FMC_LAUNCH_CHECK();
  return FMC_OK;
}

// Adjoint of layer l's last Linear + spline, recomputing the Linear from A
// (the last tanh activation, bf16 [rows_a, K]).
int tc_linear_spline_bwd(cudaStream_t st, const FlowGeom& g, const FmcFlow* f, int l, const uint16_t* A, int64_t M,
                         int64_t rows_a, const float* xa, const float* gy, float gld, float* gxa, uint16_t* graw,
                         int64_t ldg, float* bpart) {
  const int nt = g.nt(l);
  int dg, bn;
  const int n_groups = spline_groups(g.K, nt, &dg, &bn);
  const int Kd = g.w16_cols(l, g.nh);
  FMC_CHECK_ARG(ldg >= g.draw_cols(l) && ldg % 8 == 0, "graw leading dimension too small or not a multiple of 8");
  CUtensorMap ma, mb;
  int rc = make_tma_map_bf16(&ma, A, Kd, rows_a, Kd, tc::BM);
  if (rc) return rc;
  if ((rc = make_tma_map_bf16(&mb, f->theta_bf16 + g.w16g_off[l], Kd, (int64_t)n_groups * bn, Kd, bn))) return rc;
  tc::SplineBwdArgs a;
  a.bias = f->theta + g.layer_off[l] + g.lin_b(l, g.nh);
  a.xa = xa;
  a.gy = gy;
  a.gld = gld;
  a.gxa = gxa;
  a.bpart = bpart;
  a.d = g.d;
  a.nt = nt;
  a.tpar = g.tpar(l);
  a.cpar = g.cpar(l);
  const int hl = g.H[g.nh - 1];
  const double flops = 2.0 * (double)M * nt * g.P * hl;
  // A and the weights once, x / dL/dy read, dL/dx written, dL/draw in bf16
  const double bytes = (double)M * hl * 2 + (double)nt * g.P * hl * 2 + (double)M * nt * 12 +
                       (double)M * nt * g.P * 2;
  KernelTimer kt(FMC_KT_TC_SPLINE_BWD, st, flops, bytes);
#define SPL_CASE(k)                                                  \
  if (g.K == k) {                                                    \
    rc = launch_spl_bwd<k>(st, ma, mb, M, n_groups, Kd, a, graw, ldg, g.cfg);   \
  } else
  FMC_SPLINE_BINS(SPL_CASE) {
    set_error("n_bins=%d is not instantiated for the fused spline", g.K);
    return FMC_ERR_UNSUPPORTED;
  }
#undef SPL_CASE
  return rc;
}

}  // namespace fmc
