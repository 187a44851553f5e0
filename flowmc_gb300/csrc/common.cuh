// common.cuh -- shared device helpers for libflowmc (sm_103a).
//
//  * status plumbing: thread-local error text, FMC_TRY / CUDA_TRY macros
//  * Philox-4x32-10 counter-based RNG (Salmon, Moraes, Dror, Shaw,
//    "Parallel random numbers: as easy as 1, 2, 3", SC'11), with normals by
//    the Box-Muller transform (Box & Muller, Ann. Math. Stat. 29, 1958)
//  * lane-group reductions (warp shuffles)
//  * float-float ("double-single") sums after Knuth's TwoSum (TAOCP vol. 2,
//    4.2.2) for the Metropolis-Hastings log-ratio
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string>
#include "../../include/flowmc.h"

namespace fmc {

// ---------------------------------------------------------------- errors
void set_error(const char* fmt, ...);

#define FMC_CHECK_ARG(cond, ...)                 \
  do {                                           \
    if (!(cond)) {                               \
      ::fmc::set_error(__VA_ARGS__);             \
      return FMC_ERR_INVALID_ARG;                \
    }                                            \
  } while (0)

#define FMC_CHECK_SUPPORTED(cond, ...)           \
  do {                                           \
    if (!(cond)) {                               \
      ::fmc::set_error(__VA_ARGS__);             \
      return FMC_ERR_UNSUPPORTED;                \
    }                                            \
  } while (0)

// a failed runtime call also leaves the runtime's last-error state set;
// it is cleared here so that it is not reported again by the next launch
#define FMC_CUDA_TRY(expr)                                                   \
  do {                                                                       \
    cudaError_t _e = (expr);                                                 \
    if (_e != cudaSuccess) {                                                 \
      (void)cudaGetLastError();                                              \
      ::fmc::set_error("%s failed: %s (%s:%d)", #expr, cudaGetErrorString(_e), \
                       __FILE__, __LINE__);                                  \
      return FMC_ERR_CUDA;                                                   \
    }                                                                        \
  } while (0)

#define FMC_LAUNCH_CHECK()                                                   \
  do {                                                                       \
    ::fmc::count_launch();                                                   \
    cudaError_t _e = cudaGetLastError();                                     \
    if (_e != cudaSuccess) {                                                 \
      ::fmc::set_error("kernel launch failed: %s (%s:%d)",                  \
                       cudaGetErrorString(_e), __FILE__, __LINE__);          \
      return FMC_ERR_CUDA;                                                   \
    }                                                                        \
  } while (0)

int sm_count();  // cached per device
void count_launch();  // process-wide tally of kernel launches (fmc_launch_count)

// ---------------------------------------------------------------- kernel timing
// Optional per-kernel timing (fmc_kernel_timing_*): while enabled, a
// KernelTimer scope records a CUDA event pair on the launch stream around
// the launch it encloses, together with the launch's algorithmic FLOPs and
// bytes as the caller states them. On a capturing stream the pair becomes
// two event-record nodes of the graph, timed when the graph is replayed.
// The ids are the FMC_KT_* values of flowmc.h.
// launch geometry of the last launch of kernel `kid` (fmc_kernel_grid)
void note_grid(int kid, int ctas, int cluster);

struct KernelTimer {
  int slot = -1;
  bool capturing = false;
  cudaStream_t st = nullptr;
  KernelTimer(int kid, cudaStream_t stream, double flops, double bytes);
  ~KernelTimer();
  KernelTimer(const KernelTimer&) = delete;
  KernelTimer& operator=(const KernelTimer&) = delete;
};

// ---------------------------------------------------------------- Philox
// Philox-4x32 with R rounds, constants from the SC'11 paper (Table 2 and
// the Weyl key schedule). counter = 4 x u32, key = 2 x u32. R = 10 is the
// paper's recommended count; R = 7 is the smallest it reports as
// Crush-resistant (an option of the local-step kernel, off by default).
struct u32x4 { uint32_t x, y, z, w; };

template <int R>
__host__ __device__ __forceinline__ u32x4 philox4x32(u32x4 c, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    // one 32x32 -> 64-bit multiply gives both halves of each product
    const uint64_t p0 = (uint64_t)M0 * c.x, p1 = (uint64_t)M1 * c.z;
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    c = u32x4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    k0 += W0;
    k1 += W1;
  }
  return c;
}

__host__ __device__ __forceinline__ u32x4 philox4x32_10(u32x4 c, uint32_t k0, uint32_t k1) {
  return philox4x32<10>(c, k0, k1);
}

// u32 -> uniform in (0, 1]: 24 significant bits, never 0 (log finite).
__device__ __forceinline__ float u32_to_unit(uint32_t v) {
  return (float)((v >> 8) + 1u) * (1.0f / 16777216.0f);
}

// Box-Muller: two uniforms -> two independent standard normals.
__device__ __forceinline__ void box_muller(uint32_t a, uint32_t b, float& z0, float& z1) {
  const float u1 = u32_to_unit(a);
  const float u2 = u32_to_unit(b);
  // radius sqrt(-2 ln u1) as t * rsqrt(t) (two instructions instead of the
  // IEEE square root); u1 = 1 gives t = 0 and r = 0
  const float t = -2.0f * __logf(u1);
  const float r = (t > 0.f) ? t * rsqrtf(t) : 0.f;
  float s, c;
  // angle 2*pi*u2 - pi keeps the argument inside [-pi, pi] for __sincosf
  __sincosf(6.28318530717958647692f * u2 - 3.14159265358979323846f, &s, &c);
  z0 = r * c;
  z1 = r * s;
}

// Counter layout shared by every kernel: (x, y) = 64-bit stream position
// (chain index and step), z = draw slot within the step, w = stream tag.
enum : uint32_t {
  RNG_TAG_LOCAL_NORMAL = 0x4c4e0000u,
  RNG_TAG_LOCAL_UNIFORM = 0x4c550000u,
  RNG_TAG_NF_NORMAL = 0x4e4e0000u,
  RNG_TAG_NF_UNIFORM = 0x4e550000u,
  RNG_TAG_PT_EXCHANGE = 0x50580000u,
  RNG_TAG_ADAM_NOISE = 0x41440000u,
};

// SplitMix64 finaliser (Steele, Lea, Flood 2014) without the additive
// constant, so that 0 maps to 0.
__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// Device word folded into every random stream: a CUDA graph that advances it
// (fmc_rng_epoch_advance) draws fresh numbers on each replay. The library
// remembers one attached word (fmc_rng_epoch_attach); NULL or a zero word
// leaves the streams as they are.
const uint64_t* rng_epoch();

struct Rng {
  uint32_t k0, k1;     // key = seed
  uint64_t ctr_base;   // call counter, folded into the step word
  const uint64_t* epoch;
  int32_t rounds = 10; // Philox rounds: 10, or 7 where a caller opts in
  // the key this launch uses: the seed mixed with the attached epoch word
  __device__ __forceinline__ Rng at_epoch() const {
    Rng r = *this;
    if (epoch != nullptr) {
      const uint64_t e = mix64(*epoch);
      r.k0 ^= (uint32_t)e;
      r.k1 ^= (uint32_t)(e >> 32);
    }
    return r;
  }
  __device__ __forceinline__ u32x4 draw(uint64_t row, uint64_t step, uint32_t slot, uint32_t tag) const {
    const uint64_t s = step + (ctr_base << 32);
    u32x4 c{(uint32_t)row, (uint32_t)(row >> 32) ^ (uint32_t)(s >> 32), slot, tag ^ (uint32_t)s};
    return rounds == 7 ? philox4x32<7>(c, k0, k1) : philox4x32<10>(c, k0, k1);
  }
};

// ---------------------------------------------------------------- groups
// A "group" is G consecutive lanes of a warp that own one chain.
template <int G>
__device__ __forceinline__ float group_sum(float v) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o, G);
  return v;
}
template <int G>
__device__ __forceinline__ float group_max(float v) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o, G));
  return v;
}
template <int G>
__device__ __forceinline__ float group_bcast(float v, int src_lane_in_group) {
  return __shfl_sync(0xffffffffu, v, src_lane_in_group, G);
}

// ---------------------------------------------------------------- float-float
struct ff { float hi, lo; };
__device__ __forceinline__ ff two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return ff{s, e};
}
__device__ __forceinline__ ff ff_add(ff a, ff b) {
  ff s = two_sum(a.hi, b.hi);
  const float lo = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
  return two_sum(s.hi, lo);
}
__device__ __forceinline__ ff ff_neg(ff a) { return ff{-a.hi, -a.lo}; }
// exact product of two floats as float-float (FMA-based TwoProduct)
__device__ __forceinline__ ff two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  const float e = __fmaf_rn(a, b, -p);
  return ff{p, e};
}
__device__ __forceinline__ ff ff_mul_f(ff a, float b) {
  ff p = two_prod(a.hi, b);
  const float lo = __fmaf_rn(a.lo, b, p.lo);
  return two_sum(p.hi, lo);
}
// a < b where a is a float and b a float-float
__device__ __forceinline__ bool f_lt_ff(float a, ff b) {
  return (a < b.hi) || (a == b.hi && 0.0f < b.lo);
}

}  // namespace fmc
