// tc_gemm.cuh -- BF16 GEMM on the sm_100-family 5th-generation tensor cores:
//   C[M, N] = epilogue( A[M, K] . B[N, K]^T + bias )      (A, B bf16, K-major)
// with FP32 accumulation in tensor memory (TMEM).
//
// One CTA computes one 128 x BN output tile:
//   warp 0        TMA producer: cp.async.bulk.tensor loads of A and B
//                 K-chunks (64 bf16 = one 128-byte swizzle atom) into a
//                 STAGES-deep shared-memory ring (128B swizzle)
//   warp 1        TMEM allocation owner and MMA issuer: one elected thread
//                 issues tcgen05.mma.cta_group::1.kind::f16 (M=128, N=BN,
//                 K=16 per instruction, 4 per chunk) and tcgen05.commit
//                 frees each stage / signals the accumulator
//   warps 2..5    epilogue: tcgen05.ld 32x32b (one accumulator row per
//                 thread), bias, activation, conversion, global stores
// Every mbarrier wait is bounded; on expiry the kernel records an error
// code, skips the remaining work, still frees its TMEM and returns.
//
// Descriptor layouts (PTX ISA, tcgen05 "Matrix Descriptors" and
// "Instruction descriptor"): shared-memory descriptor = start>>4 [0,14),
// leading-byte-offset>>4 [16,30), stride-byte-offset>>4 [32,46), version 1
// [46,48), swizzle mode [61,64) (2 = 128B); instruction descriptor for
// kind::f16 = D format [4,6) (1 = f32), A format [7,10) and B format
// [10,13) (1 = bf16), A/B major [15], [16] (0 = K-major), N>>3 [17,23),
// M>>4 [24,29).
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include "common.cuh"
#include "gemm_tc.cuh"

namespace fmc {
namespace tc {

constexpr int BM = 128;
constexpr int BK = 64;                 // bf16 elements per 128-byte swizzle row
constexpr int kEpiWarps = 8;   // two per TMEM lane quarter
constexpr int kThreads = 64 + 32 * kEpiWarps;

// epilogue modes and arguments: see gemm_tc.cuh

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// bounded wait: try_wait suspends the thread until the phase completes or an
// implementation-defined time passes (a few microseconds), so the bound is on
// wall time (%globaltimer), not on a count of tries: gives up after one second
// and returns false.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  do {
    if (mbar_try_wait(bar, parity)) return true;
  } while (global_ns() - t0 < 1000000000ull);
  return false;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];"
      ::"r"(smem_u32(dst)), "l"((uint64_t)map), "r"(smem_u32(bar)), "r"(c0), "r"(c1)
      : "memory");
}

__device__ __forceinline__ uint64_t smem_desc_sw128(const void* p) {
  const uint64_t addr = smem_u32(p);
  uint64_t d = 0;
  d |= (addr >> 4) & 0x3FFFull;             // start address
  d |= (uint64_t)1 << 16;                   // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;         // stride byte offset: 8 rows x 128 B
  d |= (uint64_t)1 << 46;                   // descriptor version (sm_100 family)
  d |= (uint64_t)2 << 61;                   // 128-byte swizzle
  return d;
}

// MN-major operand in 128-byte swizzle: the tile is stored as K rows of 64
// MN elements (128 bytes each; one TMA box {64 MN, 64 K} = 8 KB per 64-wide MN
// block). Canonical layout ((8,8,m),(8,k)) : ((1,8,LBO),(64,SBO)) in elements:
// LBO = 8192 B between the 64-wide MN blocks, SBO = 1024 B between groups of
// eight K rows; one K = 16 step of the MMA advances the start by 2048 B.
constexpr int kMnBlockBytes = 64 * BK * 2;
__device__ __forceinline__ uint64_t smem_desc_sw128_mn(const void* p) {
  const uint64_t addr = smem_u32(p);
  uint64_t d = 0;
  d |= (addr >> 4) & 0x3FFFull;                       // start address
  d |= (uint64_t)(kMnBlockBytes >> 4) << 16;          // leading byte offset: next 64-wide MN block
  d |= (uint64_t)(1024 >> 4) << 32;                   // stride byte offset: next 8 K rows
  d |= (uint64_t)1 << 46;                             // descriptor version (sm_100 family)
  d |= (uint64_t)2 << 61;                             // 128-byte swizzle
  return d;
}

__host__ __device__ constexpr uint32_t idesc_bf16_f32(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) {
    asm volatile("" : "+r"(r[i]));   // keep every use after the wait
    v[i] = __uint_as_float(r[i]);
  }
}

// issue a 32-column TMEM load without waiting; the registers must not be
// read before tmem_wait_pin
__device__ __forceinline__ void tmem_ld32_issue(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
}

// wait for this thread's TMEM loads; every register is pinned after the wait
__device__ __forceinline__ void tmem_wait_pin(uint32_t (&r)[32]) {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) asm volatile("" : "+r"(r[i]));
}

__device__ __forceinline__ float tanh_fast(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

template <int BN, int STAGES>
struct Smem {
  static constexpr int A_BYTES = BM * BK * 2;
  static constexpr int B_BYTES = BN * BK * 2;
  static constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
  static constexpr int TOTAL = STAGES * STAGE_BYTES + 1024 /*align slack*/ + 256 /*barriers*/;
};

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// ---- TMA store of the bf16 epilogues: each epilogue warp stages a 32-row x
// 64-column block (4 KB, the 128-byte swizzle of the output tensor map: the
// 16-byte chunk c of row r sits at r*128 + ((c ^ (r & 7)) * 16)) and one lane
// stores it with cp.async.bulk.tensor; NSTG staging buffers per warp (two let
// a warp fill one block while the previous one is still being stored; one
// leaves room for a deeper operand ring).
constexpr int kStageBlockBytes = 32 * 128;
__host__ __device__ constexpr int staging_bytes(int nstg) { return kEpiWarps * nstg * kStageBlockBytes; }

__device__ __forceinline__ void st_shared_v4(uint32_t addr, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
  asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(a), "r"(b), "r"(c), "r"(d) : "memory");
}
__device__ __forceinline__ void tma_store_2d(const CUtensorMap* map, uint32_t src, int c0, int c1) {
  asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%2, %3}], [%1];"
               ::"l"((uint64_t)map), "r"(src), "r"(c0), "r"(c1)
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// at most one committed store group may still be reading shared memory
__device__ __forceinline__ void bulk_wait_read_1() { asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
// every committed store group has finished reading shared memory
__device__ __forceinline__ void bulk_wait_read_0() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// TMA store of an fp32 box (generic address of the shared-memory source)
__device__ __forceinline__ void tma_store_2d_f32(const CUtensorMap* map, uint32_t src, int c0, int c1) {
  asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%2, %3}], [%1];"
               ::"l"((uint64_t)map), "r"(src), "r"(c0), "r"(c1)
               : "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// ---- CTA pairs (tcgen05 cta_group::2). Two CTAs of a cluster share one
// 256-row MMA: each holds its 128 rows of A and half of the B rows in its own
// shared memory (at the same offsets), the even CTA issues
// tcgen05.mma.cta_group::2 for both, and each CTA's TMEM receives its own
// 128 accumulator rows over all N columns. B is read once per pair instead of
// once per CTA.
__device__ __forceinline__ uint32_t cluster_ctarank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

// shared::cluster address of the variable at shared::cta address `a` in CTA `rank`
__device__ __forceinline__ uint32_t mapa_shared(uint32_t a, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
  return r;
}

// every thread of both CTAs: arrive (release) and wait (acquire) on the
// cluster barrier (the non-aligned forms: warps need not be converged)
__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
}

// bounded wait on a barrier of this CTA that threads of the peer CTA (or the
// pair's MMAs and copies) also complete: acquire at cluster scope
__device__ __forceinline__ bool mbar_try_wait_cl(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ bool mbar_wait_cl(uint64_t* bar, uint32_t parity) {
  if (mbar_try_wait_cl(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  do {
    if (mbar_try_wait_cl(bar, parity)) return true;
  } while (global_ns() - t0 < 1000000000ull);
  return false;
}

// arrive on an mbarrier given by its shared::cluster address (either CTA)
__device__ __forceinline__ void mbar_arrive_cluster(uint32_t cl_addr) {
  asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(cl_addr) : "memory");
}

// TMA load into this CTA's shared memory whose completion is counted on an
// mbarrier of either CTA of the pair (shared::cluster address)
__device__ __forceinline__ void tma_load_2d_pair(void* dst, const CUtensorMap* map, uint32_t bar_cl, int c0, int c1) {
  asm volatile(
      "cp.async.bulk.tensor.2d.cta_group::2.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], "
      "[%2];" ::"r"(smem_u32(dst)),
      "l"((uint64_t)map), "r"(bar_cl), "r"(c0), "r"(c1)
      : "memory");
}

// M = 256 instruction descriptor of a CTA pair (each CTA: 128 rows)
__host__ __device__ constexpr uint32_t idesc_bf16_f32_pair(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(256 >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16_pair(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

// arrive on the mbarrier at this shared offset in both CTAs once every MMA
// the pair issued so far has completed
__device__ __forceinline__ void mma_commit_pair(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;" ::"r"(
          smem_u32(bar)),
      "h"((uint16_t)3)
      : "memory");
}

// Fail fast after a broken pipeline: when the device error word is already
// raised (a bounded wait of an earlier tensor-core launch expired and nobody
// cleared the word), the CTA does no work at all -- no TMEM allocation, no
// waits -- so that a run whose tensor-core pipeline broke ends within one
// wait bound instead of one bound per later launch. The decision is made by
// one thread and shared, so every thread of the CTA takes the same branch.
__device__ __forceinline__ bool tc_skip(const int* err) {
  __shared__ int s_skip;
  if (threadIdx.x == 0) s_skip = *(const volatile int*)err;
  __syncthreads();
  return s_skip != 0;
}

// the error-word check of tc_skip, made by the even CTA for the pair
__device__ __forceinline__ bool tc_skip_pair(const int* err) {
  __shared__ int s_skip;
  if (threadIdx.x == 0) s_skip = (cluster_ctarank() == 0) ? *(const volatile int*)err : 0;
  cluster_sync_all();
  int v;
  asm volatile("ld.shared::cluster.u32 %0, [%1];" : "=r"(v) : "r"(mapa_shared(smem_u32(&s_skip), 0)) : "memory");
  cluster_sync_all();   // the even CTA's word stays readable until both have read it
  return v != 0;
}

// Persistent GEMM: each CTA walks work items t = blockIdx.x, +gridDim.x, ...
// Item t is K-slice s = t % splits of tile t / splits (tile u covers rows
// (u / n_tiles) * 128 and columns (u % n_tiles) * BN); with splits > 1 the
// slices write their fp32 partial products to C + s * split_stride and the
// host reduces them. Two TMEM accumulators let the epilogue of one item
// overlap the MMAs of the next. err: device word; 1 = a wait expired.
// TSTORE (bf16 modes only): the row-major output goes through per-warp
// shared-memory staging and TMA stores on tmC ([M, n_store] bf16, box 64 x 32);
// the shared memory then holds the ring, its barriers, 768 bytes of padding
// and the staging buffers (staging_bytes(NSTG), 1024-byte aligned).
// NSTG = 2 also stages each chunk's 32 bias values in shared memory (one
// 128-byte slot per epilogue warp, broadcast reads); with NSTG = 1 the bias
// reaches the lanes by shuffles.
// PAIR (launched as clusters of 2, no split-K): a tile is 256 rows x BN
// columns computed by a CTA pair with tcgen05 cta_group::2 -- each CTA loads
// its 128 rows of A and BN / 2 rows of B (tmB's box is BN / 2 rows), the
// even CTA issues the MMAs, each CTA runs the epilogue of its own rows.
template <int BN, int STAGES, int EPI, bool TSTORE, bool PAIR = false, int NSTG = 2, int OPM = 0>
__global__ void __launch_bounds__(kThreads, 1)
    k_tc_gemm(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
              const __grid_constant__ CUtensorMap tmC, int M, int N, int K, const EpiArgs ep, void* __restrict__ C,
              int64_t ldc, int n_store, int splits, int64_t split_stride, int* err) {
  static_assert(!TSTORE || EPI == TC_EPI_TANH_BF16 || EPI == TC_EPI_DTANH_BF16, "TMA store: bf16 epilogues only");
  static_assert(!PAIR || BN % 32 == 0, "a CTA pair splits B into two multiples of 16 rows");
  static_assert(NSTG == 1 || NSTG == 2, "one or two staging buffers per warp");
  static_assert(OPM == 0 || (!PAIR && BN % 64 == 0), "MN-major operands: one-CTA tiles of whole 64-wide blocks");
  constexpr bool kBiasSmem = NSTG == 2;
  if (PAIR ? tc_skip_pair(err) : tc_skip(err)) return;
  extern __shared__ uint8_t smem_raw[];
  __shared__ __align__(16) float s_bias[kBiasSmem ? kEpiWarps : 1][32];
  constexpr int BNL = PAIR ? BN / 2 : BN;   // B rows this CTA loads per stage
  using S = Smem<BNL, STAGES>;
  uint8_t* base = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint8_t* staging = base + STAGES * S::STAGE_BYTES + 1024;
  uint64_t* full = (uint64_t*)(base + STAGES * S::STAGE_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* acc_full = empty + STAGES;      // [2]
  uint64_t* acc_empty = acc_full + 2;       // [2]
  uint64_t* mma_done = acc_empty + 2;
  uint32_t* tmem_slot = (uint32_t*)(mma_done + 1);
  volatile int* abort_flag = (volatile int*)(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nk = (K + BK - 1) / BK;
  const int nks = (nk + splits - 1) / splits;   // K chunks per slice
  const int n_tiles = (n_store + BN - 1) / BN;
  constexpr int TM = PAIR ? 2 * BM : BM;        // rows per tile
  const int m_tiles = (M + TM - 1) / TM;
  const int tiles = n_tiles * m_tiles * splits;
  const uint32_t rank = PAIR ? cluster_ctarank() : 0u;
  const int t_first = PAIR ? (int)(blockIdx.x / 2) : (int)blockIdx.x;   // work items of this CTA (pair)
  const int t_step = PAIR ? (int)(gridDim.x / 2) : (int)gridDim.x;
  // waits: the ring and accumulator-full barriers are completed by copies
  // and MMA commits (asynchronous proxy), which a CTA-scope acquire covers;
  // the accumulator-empty barrier of a pair counts the odd CTA's threads too
  // and is waited on at cluster scope (wait_cl)
  auto wait = [](uint64_t* bar, uint32_t ph) { return mbar_wait(bar, ph); };
  auto wait_cl = [](uint64_t* bar, uint32_t ph) { return PAIR ? mbar_wait_cl(bar, ph) : mbar_wait(bar, ph); };

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], (PAIR ? 2 : 1) * kEpiWarps);
    }
    mbar_init(mma_done, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    if constexpr (PAIR) {
      asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                   "r"(2 * BN));
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;");
    } else {
      asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                   "r"(2 * BN));
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if constexpr (PAIR) cluster_sync_all();   // both CTAs' barriers exist before either signals the other's
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      uint32_t it = 0;
      for (int t = t_first; t < tiles && !*abort_flag; t += t_step) {
        const int u = t / splits, sl = t - u * splits;
        const int m0 = (u / n_tiles) * TM + (int)rank * BM, n0 = (u % n_tiles) * BN + (int)rank * BNL;
        const int kb = sl * nks, ke = (kb + nks < nk) ? kb + nks : nk;
        for (int k = kb; k < ke; ++k, ++it) {
          const int s = it % STAGES;
          const uint32_t ph = (it / STAGES) & 1u;
          if (it >= (uint32_t)STAGES && !wait(&empty[s], ph ^ 1u)) {
            *abort_flag = 1;
            break;
          }
          if (*abort_flag) break;
          uint8_t* sa = base + s * S::STAGE_BYTES;
          uint8_t* sb = sa + S::A_BYTES;
          if constexpr (PAIR) {
            // both CTAs' copies count on the even CTA's barrier
            const uint32_t full_cl = mapa_shared(smem_u32(&full[s]), 0);
            if (rank == 0) mbar_expect_tx(&full[s], 2 * (S::A_BYTES + S::B_BYTES));
            tma_load_2d_pair(sa, &tmA, full_cl, k * BK, m0);
            tma_load_2d_pair(sb, &tmB, full_cl, k * BK, n0);
          } else {
            mbar_expect_tx(&full[s], S::STAGE_BYTES);
            if constexpr ((OPM & 1) != 0) {
#pragma unroll
              for (int j = 0; j < BM / 64; ++j) tma_load_2d(sa + j * kMnBlockBytes, &tmA, &full[s], m0 + 64 * j, k * BK);
            } else {
              tma_load_2d(sa, &tmA, &full[s], k * BK, m0);
            }
            if constexpr ((OPM & 2) != 0) {
#pragma unroll
              for (int j = 0; j < BN / 64; ++j) tma_load_2d(sb + j * kMnBlockBytes, &tmB, &full[s], n0 + 64 * j, k * BK);
            } else {
              tma_load_2d(sb, &tmB, &full[s], k * BK, n0);
            }
          }
        }
      }
      if (*abort_flag) {
        // let the copies still in flight land before the CTA exits (bounded;
        // a pair's copies count on the even CTA, so the odd one waits on the
        // stages' release instead)
        for (uint32_t j = it > (uint32_t)STAGES ? it - STAGES : 0; j < it; ++j) {
          if (PAIR && rank != 0)
            wait(&empty[j % STAGES], (j / STAGES) & 1u);
          else
            wait(&full[j % STAGES], (j / STAGES) & 1u);
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0 && rank == 0) {
      // bits 15 / 16 of the instruction descriptor: A / B MN-major
      const uint32_t idesc = (PAIR ? idesc_bf16_f32_pair(BN) : idesc_bf16_f32(BN)) | ((OPM & 1) ? 1u << 15 : 0u) |
                             ((OPM & 2) ? 1u << 16 : 0u);
      uint32_t it = 0;
      int local = 0;
      for (int t = t_first; t < tiles && !*abort_flag; t += t_step, ++local) {
        const int b = local & 1, use = local >> 1;
        if (use > 0 && !wait_cl(&acc_empty[b], (uint32_t)(use - 1) & 1u)) {
          *abort_flag = 1;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t d = tmem + (uint32_t)(b * BN);
        const int sl = t % splits;
        const int kb = sl * nks, ke = (kb + nks < nk) ? kb + nks : nk;
        bool stop = false;
        for (int k = kb; k < ke; ++k, ++it) {
          const int s = it % STAGES;
          const uint32_t ph = (it / STAGES) & 1u;
          if (!wait(&full[s], ph) || *abort_flag) {
            *abort_flag = 1;
            stop = true;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint8_t* sa = base + s * S::STAGE_BYTES;
          const uint8_t* sb = sa + S::A_BYTES;
          const uint64_t da = (OPM & 1) ? smem_desc_sw128_mn(sa) : smem_desc_sw128(sa);
          const uint64_t db = (OPM & 2) ? smem_desc_sw128_mn(sb) : smem_desc_sw128(sb);
          // start-address step of one K = 16 slice (16-byte units): 32 B inside a
          // K-major swizzle row, 16 rows of 128 B in an MN-major tile
          constexpr uint64_t kStepA = (OPM & 1) ? 128 : 2, kStepB = (OPM & 2) ? 128 : 2;
#pragma unroll
          for (int kk = 0; kk < BK / 16; ++kk) {
            // advance along K inside the swizzle atom: 16 bf16 = 32 bytes
            if constexpr (PAIR)
              mma_bf16_pair(d, da + (uint64_t)(kk * 2), db + (uint64_t)(kk * 2), idesc, (k > kb || kk > 0) ? 1u : 0u);
            else
              mma_bf16(d, da + kStepA * kk, db + kStepB * kk, idesc, (k > kb || kk > 0) ? 1u : 0u);
          }
          if constexpr (PAIR) mma_commit_pair(&empty[s]); else mma_commit(&empty[s]);
        }
        if (stop) break;
        if constexpr (PAIR) mma_commit_pair(&acc_full[b]); else mma_commit(&acc_full[b]);
      }
      // fires once every MMA issued so far has finished (also after an abort),
      // so the TMEM can be released safely (in both CTAs of a pair)
      if constexpr (PAIR) mma_commit_pair(mma_done); else mma_commit(mma_done);
    }
  } else {
    // epilogue warps: TMEM lane quarter = warp % 4, one accumulator row per
    // thread; the two warps of a quarter take alternate 32-column chunks
    const int q = warp & 3;
    const int half = (warp - 2) >> 2;
    const int row = q * 32 + lane;
    // vector stores only when every row start is 16-byte aligned
    const int esz = (EPI == TC_EPI_TANH_BF16 || EPI == TC_EPI_DTANH_BF16) ? 2 : 4;
    const bool vec_ok = (((uintptr_t)C & 15) == 0) && ((ldc * esz) % 16 == 0);
    const bool aux_vec = (((uintptr_t)ep.aux & 15) == 0) && ((ep.ldaux * 2) % 16 == 0);
    int blkno = 0;   // staged blocks so far (selects the staging buffer)
    int local = 0;
    const uint32_t acc_empty_cl0 = PAIR ? mapa_shared(smem_u32(&acc_empty[0]), 0) : 0u;
    const uint32_t acc_empty_cl1 = PAIR ? mapa_shared(smem_u32(&acc_empty[1]), 0) : 0u;
    for (int t = t_first; t < tiles; t += t_step, ++local) {
      const int b = local & 1, use = local >> 1;
      const int u = t / splits, sl = t - u * splits;
      const int m0 = (u / n_tiles) * TM + (int)rank * BM, n0 = (u % n_tiles) * BN;
      const int gm = m0 + row;
      if (*abort_flag || !wait(&acc_full[b], (uint32_t)use & 1u)) {
        *abort_flag = 1;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const bool row_ok = gm < M;
      const uint32_t tbase = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * BN);
      // One 32-column chunk: v = accumulator row segment, bl = bias of column
      // n0 + c0 + lane (lane-distributed, broadcast with shuffles before any
      // lane-dependent branch), av = the row's tanh activations (mode 2).
      auto chunk = [&](const uint32_t (&r)[32], int c0, float bl, const uint4 (&av)[4], int sub) {
        const int gn0 = n0 + c0;
        if (gn0 >= n_store) return;   // uniform across the warp
        float v[32];
#pragma unroll
        for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
        if (EPI == TC_EPI_TANH_BF16 || EPI == TC_EPI_BIAS_F32) {
          if constexpr (kBiasSmem) {
            // the warp's slot: lane i writes bias i, every lane reads all 32 (broadcast)
            float* sbw = s_bias[warp - 2];
            sbw[lane] = bl;
            __syncwarp();
            const float4* b4 = reinterpret_cast<const float4*>(sbw);
#pragma unroll
            for (int i = 0; i < 8; ++i) {
              const float4 bb = b4[i];
              v[4 * i] += bb.x;
              v[4 * i + 1] += bb.y;
              v[4 * i + 2] += bb.z;
              v[4 * i + 3] += bb.w;
            }
            __syncwarp();
          } else {
#pragma unroll
            for (int i = 0; i < 32; ++i) v[i] += __shfl_sync(0xffffffffu, bl, i);
          }
        }
        if (!TSTORE && !row_ok) return;
        if (EPI == TC_EPI_TANH_BF16 || EPI == TC_EPI_DTANH_BF16) {
          uint32_t packed[16];
          float y[32];
          if (EPI == TC_EPI_TANH_BF16) {
            if (gn0 + 32 <= N && row_ok) {   // the whole chunk is inside the output
#pragma unroll
              for (int i = 0; i < 32; ++i) y[i] = tanh_fast(v[i]);
            } else {
#pragma unroll
              for (int i = 0; i < 32; ++i) y[i] = (gn0 + i < N && row_ok) ? tanh_fast(v[i]) : 0.f;
            }
          } else {
            const uint16_t* hv = reinterpret_cast<const uint16_t*>(av);
#pragma unroll
            for (int i = 0; i < 32; ++i) {
              const float h = __uint_as_float((uint32_t)hv[i] << 16);
              y[i] = (gn0 + i < N && row_ok) ? v[i] * (1.f - h * h) : 0.f;
            }
          }
#pragma unroll
          for (int i = 0; i < 32; i += 2) {
            const __nv_bfloat162 hh = __floats2bfloat162_rn(y[i], y[i + 1]);
            packed[i / 2] = *reinterpret_cast<const uint32_t*>(&hh);
          }
          if (TSTORE) {
            // half `sub` of this warp's current 64-column block (zeros in rows >= M are clipped by the store)
            const uint32_t buf = smem_u32(staging) + (uint32_t)(((warp - 2) * NSTG + (blkno % NSTG)) * kStageBlockBytes);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              const int cc = sub * 4 + k;
              st_shared_v4(buf + (uint32_t)(lane * 128 + ((cc ^ (lane & 7)) << 4)), packed[4 * k], packed[4 * k + 1],
                           packed[4 * k + 2], packed[4 * k + 3]);
            }
          } else if (row_ok) {
            __nv_bfloat16* out = (__nv_bfloat16*)C + (int64_t)gm * ldc + gn0;
            if (gn0 + 32 <= n_store && vec_ok) {
              uint4* o4 = reinterpret_cast<uint4*>(out);
#pragma unroll
              for (int i = 0; i < 4; ++i)
                o4[i] = make_uint4(packed[4 * i], packed[4 * i + 1], packed[4 * i + 2], packed[4 * i + 3]);
            } else {
              uint16_t* o16 = reinterpret_cast<uint16_t*>(out);
#pragma unroll
              for (int i = 0; i < 32; ++i)
                if (gn0 + i < n_store) o16[i] = (i & 1) ? (uint16_t)(packed[i / 2] >> 16) : (uint16_t)packed[i / 2];
            }
          }
        } else if (row_ok) {
          // fp32 output row: gm, or through the row map of a padded operand
          // (splits == 1; the split-K reduction applies it otherwise)
          int64_t orow = gm;
          if (ep.rmap_grp > 0 && splits == 1) {
            const int t = gm / ep.rmap_grp, p = gm - t * ep.rmap_grp;
            if (p >= ep.rmap_keep) return;
            orow = (int64_t)t * ep.rmap_keep + p;
          }
          float* out = (float*)C + sl * split_stride + orow * ldc + gn0;
          if (gn0 + 32 <= n_store && vec_ok) {
            float4* o4 = reinterpret_cast<float4*>(out);
#pragma unroll
            for (int i = 0; i < 8; ++i) o4[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
          } else {
            const int lim = n_store - gn0 < 32 ? n_store - gn0 : 32;
#pragma unroll
            for (int i = 0; i < 32; ++i)
              if (i < lim) out[i] = v[i];
          }
        }
      };
      // operands of chunk c0 that come from global memory, loaded ahead
      auto prefetch = [&](int c0, float& bl, uint4 (&av)[4]) {
        const int j = n0 + c0 + lane;
        if (EPI == TC_EPI_TANH_BF16 || EPI == TC_EPI_BIAS_F32) bl = (j < N) ? __ldg(ep.bias + j) : 0.f;
        if (EPI == TC_EPI_DTANH_BF16) {
          const int gn0 = n0 + c0;
          const uint16_t* ar = ep.aux + (int64_t)gm * ep.ldaux + gn0;
          if (row_ok && aux_vec && gn0 + 32 <= N) {
            const uint4* a4 = reinterpret_cast<const uint4*>(ar);
#pragma unroll
            for (int i = 0; i < 4; ++i) av[i] = __ldg(a4 + i);
          } else {
            uint16_t* hv = reinterpret_cast<uint16_t*>(av);
#pragma unroll
            for (int i = 0; i < 32; ++i) hv[i] = (row_ok && gn0 + i < N) ? ar[i] : (uint16_t)0;
          }
        }
      };
      // software pipeline over this warp's NCH 32-column chunks: the TMEM
      // load and global operands of chunk i+1 are in flight while chunk i is
      // processed; the accumulator goes back to the MMA warp as soon as its
      // last chunk is in registers. Chunk order: alternate 32-column chunks of
      // the two warps of a quarter, or with TSTORE whole 64-column blocks
      // (warp `half` takes blocks half, half + 2, ...).
      constexpr int NCH = BN / 64;
      auto col_of = [&](int i) { return TSTORE ? (half + 2 * (i >> 1)) * 64 + 32 * (i & 1) : half * 32 + 64 * i; };
      uint32_t ra[32], rb[32];
      float bl_cur = 0.f, bl_nxt = 0.f;
      uint4 av_cur[4], av_nxt[4];
      tmem_ld32_issue(tbase + (uint32_t)col_of(0), ra);
      prefetch(col_of(0), bl_nxt, av_nxt);
#pragma unroll
      for (int i = 0; i < NCH; ++i) {
        const int c0 = col_of(i);
        uint32_t(&cur)[32] = (i & 1) ? rb : ra;
        uint32_t(&nxt)[32] = (i & 1) ? ra : rb;
        bl_cur = bl_nxt;
#pragma unroll
        for (int k = 0; k < 4; ++k) av_cur[k] = av_nxt[k];
        tmem_wait_pin(cur);
        if (i + 1 < NCH) {
          tmem_ld32_issue(tbase + (uint32_t)col_of(i + 1), nxt);
          prefetch(col_of(i + 1), bl_nxt, av_nxt);
        } else {
          // this warp's TMEM lanes of buffer b are read: release them to the
          // MMA warp (the even CTA's, for a pair)
          asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
          __syncwarp();
          if (lane == 0) {
            if constexpr (PAIR)
              mbar_arrive_cluster(b ? acc_empty_cl1 : acc_empty_cl0);
            else
              mbar_arrive(&acc_empty[b]);
          }
        }
        // uniform: a 64-column block inside the output, of a CTA with rows
        // inside it (the odd CTA of the last pair can lie wholly past row M)
        const bool blk_live = n0 + (c0 & ~63) < n_store && m0 < M;
        if (TSTORE && (i & 1) == 0 && blk_live) {
          // the staging buffer about to be filled was last used NSTG blocks ago
          if (lane == 0) {
            if constexpr (NSTG == 2)
              bulk_wait_read_1();
            else
              bulk_wait_read_0();
          }
          __syncwarp();
        }
        chunk(cur, c0, bl_cur, av_cur, i & 1);
        if (TSTORE && (i & 1) == 1 && blk_live) {
          fence_proxy_async_smem();
          __syncwarp();
          if (EPI == TC_EPI_DTANH_BF16 && ep.colpart != nullptr) {
            // column sums of the staged 32 x 64 block: lane l takes columns
            // 2l, 2l+1 (one 4-byte word per row: the 32 lanes cover a row's
            // 128 bytes, no bank conflicts); rows >= M were staged as zeros
            const uint32_t buf =
                smem_u32(staging) + (uint32_t)(((warp - 2) * NSTG + (blkno % NSTG)) * kStageBlockBytes);
            float s0 = 0.f, s1 = 0.f;
#pragma unroll 8
            for (int r = 0; r < 32; ++r) {
              uint32_t v;
              const uint32_t addr = buf + (uint32_t)(r * 128 + (((lane >> 2) ^ (r & 7)) << 4) + ((lane & 3) << 2));
              asm volatile("ld.shared.b32 %0, [%1];" : "=r"(v) : "r"(addr));
              s0 += __uint_as_float(v << 16);
              s1 += __uint_as_float(v & 0xffff0000u);
            }
            const int col = n0 + (c0 & ~63) + 2 * lane;
            float* dst = ep.colpart + (int64_t)(m0 / 32 + q) * ep.ldpart;
            if (col < N) dst[col] = s0;
            if (col + 1 < N) dst[col + 1] = s1;
          }
          if (lane == 0) {
            tma_store_2d(&tmC, smem_u32(staging) + (uint32_t)(((warp - 2) * NSTG + (blkno % NSTG)) * kStageBlockBytes),
                         n0 + (c0 & ~63), m0 + q * 32);
            bulk_commit();
          }
          ++blkno;
        }
      }
    }
  }
  // staged stores must finish reading shared memory before the CTA exits
  if (TSTORE && warp >= 2 && lane == 0) bulk_wait_all();
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    if (lane == 0) wait_cl(mma_done, 0);
    __syncwarp();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if constexpr (PAIR)
      asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * BN));
    else
      asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * BN));
  }
  if (threadIdx.x == 0 && *abort_flag) atomicExch(err, 1);
  // neither CTA of a pair leaves while the other may still signal its barriers
  if constexpr (PAIR) cluster_sync_all();
}

}  // namespace tc
}  // namespace fmc
