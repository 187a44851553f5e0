/*
 * flowmc.h -- C ABI of libflowmc, the sm_103a (GB300) implementation of
 * flowMC's sampling hot path.
 *
 * Conventions (every entry point):
 *   - returns an int status (FMC_OK = 0); on failure fmc_last_error() gives a
 *     thread-local message. No entry point aborts, traps or asserts.
 *   - every pointer is a DEVICE pointer owned by the caller, unless the
 *     comment says "host". The library allocates no device memory.
 *   - work is enqueued on `stream` (a cudaStream_t passed as void*); nothing
 *     synchronises the host unless the comment says so.
 *   - float32 row-major arrays; chain buffers use flowMC's layout
 *     positions[n_chains, buf_len, n_dim], log_prob/acceptance[n_chains, buf_len].
 *
 * Reference files are cited as they appear in flowMC v0.4.5 (src/flowMC/...).
 */
#ifndef FLOWMC_H
#define FLOWMC_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FMC_ABI_VERSION 1

#if defined(__GNUC__)
#define FMC_API __attribute__((visibility("default")))
#else
#define FMC_API
#endif

/* ---- status codes ---------------------------------------------------- */
enum {
  FMC_OK = 0,
  FMC_ERR_INVALID_ARG = 1,    /* bad pointer / shape / value            */
  FMC_ERR_UNSUPPORTED = 2,    /* shape or option this build cannot run  */
  FMC_ERR_CUDA = 3,           /* a CUDA runtime call failed             */
  FMC_ERR_TIMEOUT = 4,        /* a bounded device wait ran out          */
  FMC_ERR_NONFINITE = 5       /* non-finite value where one is forbidden */
};

/* ---- target log-densities (replace the user's JAX callable) --------- */
/* A registered device target: value and analytic gradient in the kernels.
 * Replaces `LogPDF.__call__` (resource/logPDF.py:225-226) plus
 * `jax.value_and_grad(logpdf)` (resource/kernel/MALA.py:59, HMC.py:73-78). */
enum {
  FMC_TARGET_DIAG_GAUSSIAN = 0, /* -0.5 sum_j (x_j-mean_j)^2 * inv_var_j + scalars[0]   */
  FMC_TARGET_DUAL_MOON = 1,     /* -0.5((|x|-s0)/s1)^2 + logsumexp_{+-}(-0.5((x0 -+ s2)/s3)^2) */
  FMC_TARGET_GAUSS_MIXTURE = 2, /* logsumexp_k(logw_k - 0.5 sum_j (x_j-mean_kj)^2 inv_var_kj) */
  FMC_TARGET_ROSENBROCK = 3,    /* -sum_{i<d-1} (s1-x_i)^2/s0 + s2 (x_{i+1}-x_i^2)^2           */
  FMC_TARGET_DENSE_GAUSSIAN = 4 /* -0.5 (x-mean)^T P (x-mean) + scalars[0]                     */
};

typedef struct FmcTarget {
  int32_t kind;          /* FMC_TARGET_*                                   */
  int32_t n_dim;
  int32_t n_comp;        /* mixture components (GAUSS_MIXTURE)             */
  int32_t reserved;
  const float* mean;     /* [n_dim] or [n_comp, n_dim]; may be NULL (zero) */
  const float* inv_var;  /* [n_dim] or [n_comp, n_dim]; may be NULL (one)  */
  const float* log_w;    /* [n_comp]: log weight + log normaliser per component */
  const float* precision;/* [n_dim, n_dim] (DENSE_GAUSSIAN)                */
  float scalars[8];      /* kind-specific constants, see the enum above    */
} FmcTarget;

/* ---- local kernels ---------------------------------------------------- */
enum { FMC_KERNEL_MALA = 0, FMC_KERNEL_HMC = 1, FMC_KERNEL_GRW = 2 };

typedef struct FmcLocalParams {
  int32_t kind;               /* FMC_KERNEL_*                                    */
  int32_t n_leapfrog;         /* HMC: rows-2 of the leapfrog table (HMC.py:25-27) */
  float step_size;            /* MALA dt, HMC epsilon, GRW sigma                 */
  int32_t lanes_per_chain;    /* 0 = choose; else 1,2,4,8,16,32 (autotuner)      */
  const float* momentum_scale;/* HMC: [n_dim] = diag(cholesky(inv(M)))   or NULL = 1 */
  const float* metric_colsum; /* HMC: [n_dim] = sum_i M[i, j]            or NULL = 1 */
} FmcLocalParams;

/* Run `n_steps` steps of a local kernel for every chain in one persistent
 * launch, keeping each chain's position, log-density and gradient on-chip,
 * with in-kernel Philox-4x32-10 noise (or explicit noise) and the MH accept
 * fused in, and write every `thinning`-th step straight into the buffers.
 *
 * Replaces TakeSerialSteps.sample (strategy/take_steps.py:164-180) with
 * MALA.kernel (resource/kernel/MALA.py:26-89), HMC.kernel (HMC.py:98-151)
 * or GaussianRandomWalk.kernel (Gaussian_random_walk.py:25-61) as the scan
 * body, plus the thinning and Buffer.update_buffer writes of
 * TakeSteps.__call__ (take_steps.py:134-143, buffers.py:32-41).
 *
 *   x0        [n_chains, n_dim]   initial positions
 *   lp0       [n_chains] incoming log-densities, or NULL = logpdf(x0) as in
 *             TakeSerialSteps (take_steps.py:177). HMC and GRW use the
 *             incoming value (HMC.py:137, Gaussian_random_walk.py:57); MALA
 *             recomputes it (MALA.py:59).
 *   noise     [n_chains, n_steps, n_dim] standard normals, or NULL (Philox)
 *   unif      [n_chains, n_steps]  uniforms in (0,1], or NULL (Philox)
 *   out_pos   [n_chains, buf_len, n_dim], out_logp/out_acc [n_chains, buf_len]
 *             rows start..start+ceil(n_steps/thinning)-1 are written, with
 *             start = min(cursor, buf_len - ceil(n_steps/thinning)) (the
 *             clamping of jax.lax.dynamic_update_slice).
 *   x_last    [n_chains, n_dim]  position of the last written row
 *   lp_last   [n_chains]         its log-density
 */
FMC_API int fmc_local_steps(const FmcTarget* target, const FmcLocalParams* params,
                    const float* x0, const float* lp0, int32_t n_chains, int32_t n_steps,
                    int32_t thinning, uint64_t seed, uint64_t counter,
                    const float* noise, const float* unif,
                    float* out_pos, float* out_logp, float* out_acc,
                    int64_t buf_len, int64_t cursor,
                    float* x_last, float* lp_last, void* stream);

/* Evaluate a registered target (value and gradient) on a batch.
 * Replaces jax.vmap(jax.value_and_grad(LogPDF)) (resource/logPDF.py:225-226).
 *   x [n, n_dim] -> logp [n], grad [n, n_dim] (grad may be NULL). */
FMC_API int fmc_target_value_grad(const FmcTarget* target, const float* x, int64_t n,
                          float* logp, float* grad, void* stream);

/* ---- library --------------------------------------------------------- */
FMC_API const char* fmc_last_error(void);
FMC_API int fmc_version(void);               /* FMC_ABI_VERSION */
/* Number of SMs of the current device (host call, synchronous). */
FMC_API int fmc_device_sm_count(int32_t* out);

#ifdef __cplusplus
}
#endif
#endif /* FLOWMC_H */
