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

#define FMC_ABI_VERSION 3

#if defined(__GNUC__)
#define FMC_API __attribute__((visibility("default")))
#else
#define FMC_API
#endif

/* ---- status codes ---------------------------------------------------- */
enum {
  FMC_OK = 0,
  FMC_ERR_INVALID_ARG = 1,    /* bad pointer / shape / value            */
  FMC_ERR_UNSUPPORTED = 2,    /* shape or option the library does not run */
  FMC_ERR_CUDA = 3,           /* a CUDA runtime call failed             */
  FMC_ERR_TIMEOUT = 4,        /* a bounded device wait ran out          */
  FMC_ERR_NONFINITE = 5       /* non-finite value where one is forbidden */
};

/* ---- target log-densities (replace the user's JAX callable) --------- */
/* A registered device target: value and analytic gradient in the kernels.
 * Replaces `LogPDF.__call__` (resource/logPDF.py:60-61) plus
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
  int32_t lanes_per_chain;    /* 0 = default for n_dim; else 4, 8, 16 or 32 lanes  */
  const float* momentum_scale;/* HMC: [n_dim] = diag(cholesky(inv(M)))   or NULL = 1 */
  const float* metric_colsum; /* HMC: [n_dim] = sum_i M[i, j]            or NULL = 1 */
  const float* momentum_chol; /* HMC with a dense M: [n_dim, n_dim] row-major
                                 cholesky(inv(M)) (momentum xi @ L^T), or NULL
                                 (diagonal: momentum_scale)                     */
  int32_t philox_rounds;      /* in-kernel noise: 0 or 10 = Philox-4x32-10; 7 =
                                 Philox-4x32-7 (fewer instructions, another
                                 stream; Salmon et al. report it Crush-resistant) */
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

/* ---- parallel tempering (strategy/parallel_tempering.py) ------------- */
/* Tempered local steps: ParallelTempering._ensemble_step
 * (parallel_tempering.py:250-289) for every chain, i.e. n_steps of the local
 * kernel for each of the n_chains * n_temps (chain, temperature) rows on
 * TemperedPDF.tempered_log_pdf (resource/logPDF.py:106-108):
 *   (1 / temperatures[t]) * log L(x) + log prior(x).
 * The log-density at x0 is recomputed (parallel_tempering.py:236-238); no
 * per-step rows are stored (the reference keeps only the last state).
 *   x0           [n_chains, n_temps, n_dim]  row c * n_temps + t
 *   temperatures [n_temps] device array (n_temps <= 64)
 *   prior_mean, prior_inv_var  [n_dim] a diagonal Gaussian log prior
 *                -0.5 sum (x - m)^2 iv + prior_const, or both NULL = 0
 *   noise        [n_chains * n_temps, n_steps, n_dim] or NULL (Philox)
 *   unif         [n_chains * n_temps, n_steps] or NULL (Philox)
 *   x_last       [n_chains * n_temps, n_dim], lp_last [n_chains * n_temps]
 *                (tempered log-density)
 *   acc_count    [n_chains * n_temps] accepted steps, or NULL */
FMC_API int fmc_pt_local_steps(const FmcTarget* target, const FmcLocalParams* params, const float* x0,
                               int32_t n_chains, int32_t n_temps, const float* temperatures,
                               const float* prior_mean, const float* prior_inv_var, float prior_const,
                               int32_t n_steps, uint64_t seed, uint64_t counter, const float* noise,
                               const float* unif, float* x_last, float* lp_last, float* acc_count,
                               void* stream);

/* Exchange sweep: ParallelTempering._exchange (parallel_tempering.py:291-398)
 * for every chain. log L (untempered, no prior) at each temperature's
 * position, then for i = 0 .. n_temps-2 in order: swap positions i and i+1
 * iff log u < (1/T[i+1] - 1/T[i]) * (lp[i] - lp[i+1]).
 *   x          [n_chains, n_temps, n_dim] positions (not modified)
 *   unif       [n_chains, n_temps - 1] uniforms, or NULL (Philox)
 *   out_first  [n_chains, n_dim]  the temperature-1 position after the sweep
 *   out_rest   [n_chains, n_temps - 1, n_dim] the others, or NULL (not
 *              written: the reference keeps them only while training,
 *              parallel_tempering.py:123-132)
 *   out_logp   [n_chains, n_temps] log L after the sweep, or NULL
 *   out_acc    [n_chains, n_temps - 1] swap flags, or NULL
 *   acc_pairs  [n_temps - 1] int32 swaps accepted per pair (zeroed first) */
FMC_API int fmc_pt_exchange(const FmcTarget* target, const float* x, int32_t n_chains, int32_t n_temps,
                            const float* temperatures, uint64_t seed, uint64_t counter, const float* unif,
                            float* out_first, float* out_rest, float* out_logp, float* out_acc,
                            int32_t* acc_pairs, void* stream);

/* ParallelTempering._adapt_temperature (parallel_tempering.py:400-436) from
 * the swap counts of fmc_pt_exchange; out may alias temperatures. */
FMC_API int fmc_pt_adapt_temperatures(const float* temperatures, const int32_t* acc_pairs, int32_t n_chains,
                                      int32_t n_temps, float* out_temperatures, void* stream);

/* ---- RealNVP flow (resource/model/nf_model/realNVP.py) --------------- */
/* RealNVP(n_features, n_layers, n_hidden): per layer a MaskedCouplingLayer
 * around MLPAffine(scale_MLP, shift_MLP, dt), each MLP [d, H, d] with relu
 * (realNVP.py:120-228, common.py:127-208). theta packs, per layer:
 *   W1 [2H, d] (rows 0..H-1 the scale MLP's first Linear, H..2H-1 the
 *   shift MLP's), b1 [2H], W2s [d, H], b2s [d], W2t [d, H], b2t [d]
 * (Equinox Linear layout [out, in]). aux [2d + 2 + n_layers * d]: data_mean,
 * diag(data_cov), the base Gaussian's covariance scale, 1, then the coupling
 * masks as floats (optax's weight decay reaches them: they are float leaves
 * of the reference model). */
typedef struct FmcRealNVP {
  int32_t n_dim;
  int32_t n_layers;
  int32_t n_hidden;
  float dt;                          /* MLPAffine dt (1)                     */
  float* theta;
  float* aux;
} FmcRealNVP;

FMC_API int fmc_rnvp_layout(const FmcRealNVP* flow, int64_t* n_params, int64_t* n_aux);
/* workspace bytes for n rows; mode 0: forward / inverse / log_prob / sample,
 * 1: loss + gradient */
FMC_API int fmc_rnvp_workspace_size(const FmcRealNVP* flow, int64_t n, int32_t mode, size_t* bytes);
/* RealNVP.forward / inverse (realNVP.py:180-207): y and the summed log-det
 * [n] (inverse: layers in reverse order, negative log-det); no
 * standardisation. y may alias x. */
FMC_API int fmc_rnvp_forward(const FmcRealNVP* flow, const float* x, int64_t n, float* y, float* logdet,
                             void* ws, size_t ws_bytes, void* stream);
FMC_API int fmc_rnvp_inverse(const FmcRealNVP* flow, const float* y, int64_t n, float* x, float* logdet,
                             void* ws, size_t ws_bytes, void* stream);
/* RealNVP.log_prob (realNVP.py:215-222): standardise with data_mean /
 * diag(data_cov), forward, plus the standard normal log-density. */
FMC_API int fmc_rnvp_log_prob(const FmcRealNVP* flow, const float* x, int64_t n, float* logp, void* ws,
                              size_t ws_bytes, void* stream);
/* RealNVP.sample (realNVP.py:209-213): base normals z [n, d] (or Philox
 * when NULL) scaled by the base covariance, inverse, de-standardised. */
FMC_API int fmc_rnvp_sample(const FmcRealNVP* flow, uint64_t seed, uint64_t counter, const float* z, int64_t n,
                            float* out, void* ws, size_t ws_bytes, void* stream);
/* loss = -mean(log_prob(x)) and its gradient w.r.t. theta (NFModel.loss_fn,
 * nf_model/base.py:98-100) with a hand-written backward. */
FMC_API int fmc_rnvp_loss_grad(const FmcRealNVP* flow, const float* x, int64_t n, float* loss, float* grad,
                               void* ws, size_t ws_bytes, void* stream);

/* ---- pre-sampling optimisation (strategy/optimization.py) ------------ */
/* AdamOptimization.optimize (optimization.py:85-164) for every chain: n_steps
 * of optax.adam(learning_rate) (b1 0.9, b2 0.999, eps 1e-8) on -log p(x),
 * the gradient multiplied by (1 + xi * noise_level) with one standard normal
 * xi per chain-step, then clipped to [lower, upper] (projection_box).
 *   x0 [n_chains, n_dim]; lower / upper [n_dim] or NULL (unbounded);
 *   noise [n_chains, n_steps] normals or NULL (Philox);
 *   x_out [n_chains, n_dim]; lp_out [n_chains] log p(x_out) or NULL. */
FMC_API int fmc_adam_optimize(const FmcTarget* target, const float* x0, int32_t n_chains, int32_t n_steps,
                              float learning_rate, float noise_level, const float* lower, const float* upper,
                              uint64_t seed, uint64_t counter, const float* noise, float* x_out, float* lp_out,
                              void* stream);

/* Many dense-Gaussian targets of uneven dimension (1..256) in ONE persistent
 * launch: n_steps of MALA or HMC (identity mass) for every chain of every
 * target, chain tiles pulled by CTAs from an atomic work counter. The local
 * steps of TakeSerialSteps (strategy/take_steps.py:156-180) with MALA.kernel /
 * HMC.kernel (resource/kernel/MALA.py:26-89, HMC.py:98-151), batched across
 * targets. Host arrays (length n_targets): targets, n_chains, step_sizes,
 * noise/unif (device pointers, each may be NULL; or the array pointer NULL
 * for Philox), out_pos/out_logp/out_acc (device pointers to each target's
 * buffers [n_chains_t, buf_len, d_t] / [n_chains_t, buf_len]).
 * x0, x_last: [sum_t n_chains_t, 256] (row stride 256, target t's chains
 * from row sum_{u<t} n_chains_u); lp_last [sum_t n_chains_t]. */
FMC_API int fmc_batched_workspace_size(int32_t n_targets, int64_t total_chains, size_t* bytes);
FMC_API int fmc_batched_dense_local_steps(const FmcTarget* targets, int32_t n_targets, const int32_t* n_chains,
                                          const FmcLocalParams* params, const float* step_sizes, const float* x0,
                                          int32_t n_steps, int32_t thinning, uint64_t seed, uint64_t counter,
                                          const float* const* noise, const float* const* unif,
                                          float* const* out_pos, float* const* out_logp, float* const* out_acc,
                                          int64_t buf_len, int64_t cursor, float* x_last, float* lp_last,
                                          void* ws, size_t ws_bytes, void* stream);

/* Evaluate a registered target (value and gradient) on a batch.
 * Replaces jax.vmap(jax.value_and_grad(LogPDF)) (resource/logPDF.py:60-61).
 *   x [n, n_dim] -> logp [n], grad [n, n_dim] (grad may be NULL). */
FMC_API int fmc_target_value_grad(const FmcTarget* target, const float* x, int64_t n,
                          float* logp, float* grad, void* stream);


/* ---- MaskedCouplingRQSpline flow ------------------------------------- */
/* Model of resource/model/nf_model/rqSpline.py:364-504. Layer l is
 *   ScalarAffine(scale_l, shift_l) on all coordinates (common.py:211-240),
 *   then an RQ-spline coupling whose mask is (j + l) % 2: coordinates with
 *   (j + l) odd condition the MLP, the others are transformed
 *   (rqSpline.py:427-440, common.py:127-168).
 * Parameters live in ONE flat float32 vector `theta`; per layer, in order:
 *   scale, shift,
 *   W_0 [H_0, n_c(l)], b_0 [H_0],            (first Linear, conditioning columns only)
 *   W_i [H_i, H_{i-1}], b_i [H_i]  (i < n_hidden),
 *   W_o [n_t(l)*P, H_last], b_o [n_t(l)*P]   (last Linear, transformed-dim rows only)
 * with P = 3*n_bins+1, n_c(l) = #{j < d : (j+l) odd}, n_t(l) = d - n_c(l).
 * The reference's first-layer columns for transformed coordinates multiply
 * zeros and its last-layer rows for conditioning coordinates are masked out
 * (common.py:155-157), so they never influence a result; fmc_flow_layout
 * gives the packing. `aux` holds the float leaves the reference keeps but
 * never trains: aux[0:d] data_mean, aux[d:2d] diag(data_cov), aux[2d] the
 * base Gaussian's covariance scale c (cov = c I), aux[2d+1] the product of
 * weight-decay factors applied to the unused (packed-out) parameters. */
enum { FMC_PREC_FP32 = 0, FMC_PREC_BF16 = 1 };

#define FMC_MAX_HIDDEN 4
#define FMC_MAX_LAYERS 64

typedef struct FmcFlow {
  int32_t n_dim;
  int32_t n_layers;
  int32_t n_hidden;                  /* number of hidden Linear+tanh layers (>= 1) */
  int32_t n_bins;
  int32_t hidden[FMC_MAX_HIDDEN];
  float range_min, range_max;        /* spline range (-10, 10)            */
  float min_bin_size, min_knot_slope;/* 1e-4, 1e-4 (rqSpline.py:299-300)   */
  int32_t precision;                 /* FMC_PREC_FP32 or FMC_PREC_BF16      */
  int32_t gemm_bn;                   /* BF16 hidden-layer GEMM tile width:
                                        0 = library choice (256 for outputs
                                        wider than 128 columns, else 128),
                                        or 128 / 256 (an autotuner's pick) */
  int32_t tile_rows;                 /* rows per tensor-core tile of the BF16
                                        flow kernels (fused last Linear +
                                        spline, hidden-layer GEMMs): 0 or
                                        128 = one CTA per tile (the library
                                        choice), 256 = a CTA pair (tcgen05
                                        cta_group::2) per tile where the
                                        tile width allows (an autotuner's
                                        pick) */
  int32_t gemm_stages;               /* BF16 hidden-layer GEMMs with K >= 256
                                        on one-CTA 256-column tiles: 0 or 4 =
                                        a 4-stage operand ring and one output
                                        staging buffer per epilogue warp (the
                                        library choice), 3 = three stages,
                                        two staging buffers and the bias in
                                        shared memory (an autotuner's pick);
                                        the outputs are identical */
  int32_t wgrad_splits;              /* BF16 training: K (batch) slices of
                                        the weight-gradient GEMMs, 0 = the
                                        library choice (fill the SMs), else
                                        1..32 (an autotuner's pick; the slice
                                        sums are added in a fixed order) */
  float* theta;                      /* [n_params] float32 master weights   */
  uint16_t* theta_bf16;              /* [n_params] bf16 shadow (BF16 mode)   */
  float* aux;                        /* [2*n_dim + 2], see above             */
} FmcFlow;

/* Number of parameters and per-layer offsets into theta
 * (layer_offsets[n_layers+1], host array). */
FMC_API int fmc_flow_layout(const FmcFlow* flow, int64_t* n_params, int64_t* layer_offsets);

/* Bytes of workspace the flow entry points need for n rows (host call).
 * mode 0: log_prob / forward / inverse / sample;  1: loss + gradient. */
FMC_API int fmc_flow_workspace_size(const FmcFlow* flow, int64_t n, int32_t mode, size_t* bytes);

/* BF16 mode: theta_bf16 holds each Linear weight as a zero-padded bf16 block
 * [round_up(out, 256), round_up(in, 64)], layer by layer, followed by the
 * transposed blocks [round_up(in, 256), round_up(out, 64)] the training
 * backward reads (n_elems elements in total). fmc_flow_sync_bf16 refreshes it
 * from theta (after loading or updating parameters). */
FMC_API int fmc_flow_bf16_size(const FmcFlow* flow, int64_t* n_elems);
FMC_API int fmc_flow_sync_bf16(const FmcFlow* flow, void* stream);

/* MaskedCouplingRQSpline.forward for a batch (rqSpline.py:450-468):
 * x [n, d] -> y [n, d], logdet [n]. No standardisation. */
FMC_API int fmc_flow_forward(const FmcFlow* flow, const float* x, int64_t n, float* y, float* logdet,
                             void* ws, size_t ws_bytes, void* stream);

/* MaskedCouplingRQSpline.inverse (rqSpline.py:470-488), the reference's
 * in-layer order: ScalarAffine inverse first, then the spline inverse. */
FMC_API int fmc_flow_inverse(const FmcFlow* flow, const float* z, int64_t n, float* x, float* logdet,
                             void* ws, size_t ws_bytes, void* stream);

/* MaskedCouplingRQSpline.log_prob (rqSpline.py:498-504):
 * x [n, d] (data space) -> logp [n]. */
FMC_API int fmc_flow_log_prob(const FmcFlow* flow, const float* x, int64_t n, float* logp,
                              void* ws, size_t ws_bytes, void* stream);

/* MaskedCouplingRQSpline.sample (rqSpline.py:490-496): base normals from
 * Philox(seed, counter) or from z [n, d] when non-NULL -> x [n, d]. */
FMC_API int fmc_flow_sample(const FmcFlow* flow, uint64_t seed, uint64_t counter, const float* z,
                            int64_t n, float* x, void* ws, size_t ws_bytes, void* stream);

/* NFModel.loss_fn value and gradient (nf_model/base.py:98-100, 122):
 * loss = -mean(log_prob(x)) over x [n, d]; grad [n_params] (overwritten)
 * in theta's layout. Hand-written backward with the coupling activations
 * recomputed; loss written to *loss (device scalar). */
FMC_API int fmc_flow_loss_grad(const FmcFlow* flow, const float* x, int64_t n, float* loss, float* grad,
                               void* ws, size_t ws_bytes, void* stream);

/* ---- NFProposal global step ----------------------------------------------- */
/* NFProposal.kernel (resource/kernel/NF_proposal.py:27-172) under
 * TakeGroupSteps (strategy/take_steps.py:191-206) for every chain: n_steps
 * flow proposals per chain (base normals from Philox or z [n_chains,
 * n_steps, d]), their flow log_prob (forward pass) and target log-density,
 * and the sequential independent-MH scan with uniforms from Philox or unif
 * [n_chains, n_steps], writing thinned rows into the buffers like
 * fmc_local_steps. x_last/lp_last: the last written row. */
FMC_API int fmc_nf_workspace_size(const FmcFlow* flow, int32_t n_chains, int32_t n_steps, size_t* bytes);
FMC_API int fmc_nf_global_steps(const FmcFlow* flow, const FmcTarget* target, const float* x0, int32_t n_chains,
                                int32_t n_steps, int32_t thinning, uint64_t seed, uint64_t counter,
                                const float* z, const float* unif, float* out_pos, float* out_logp,
                                float* out_acc, int64_t buf_len, int64_t cursor, float* x_last, float* lp_last,
                                void* ws, size_t ws_bytes, void* stream);

/* The accept scan of the NF global step (NF_proposal.py:91-126) over
 * proposals a flow made elsewhere (a RealNVP, say): props [n_chains *
 * n_steps, n_dim] (row c * n_steps + s), lnf [n_chains * n_steps +
 * n_chains] their flow log-densities followed by those of x0's rows; the
 * rest as fmc_nf_global_steps. */
FMC_API int fmc_nf_accept(const FmcTarget* target, const float* x0, int32_t n_chains, int32_t n_steps,
                          int32_t thinning, uint64_t seed, uint64_t counter, const float* props, const float* lnf,
                          const float* unif, float* out_pos, float* out_logp, float* out_acc, int64_t buf_len,
                          int64_t cursor, float* x_last, float* lp_last, void* stream);

/* ---- training (NFModel.train / TrainModel without host syncs) ---------- */
/* optax.chain(clip_by_global_norm(max_norm), adamw(lr, b1, b2, eps,
 * weight_decay)) then apply_updates (resource/optimizer.py:19-22,
 * nf_model/base.py:123-124). Defaults of the reference: b1 = 0.9 (the
 * Optimizer's momentum), b2 = 0.999, eps = 1e-8, weight_decay = 1e-4,
 * max_norm = 1. */
typedef struct FmcAdamParams {
  float lr, b1, b2, eps, weight_decay, max_norm;
} FmcAdamParams;

FMC_API int fmc_adamw_workspace_size(size_t* bytes);
/* One update of theta [n] (and its bf16 shadow when non-NULL) from grad [n]
 * with moments m, v [n]; *count is optax's step count (device int32,
 * incremented). aux [n_aux] are float leaves with zero gradient: they get the
 * weight decay only. */
FMC_API int fmc_adamw_step(float* theta, uint16_t* theta_bf16, const float* grad, float* m, float* v, int64_t n,
                           float* aux, int32_t n_aux, int32_t* count, const FmcAdamParams* params, void* ws,
                           size_t ws_bytes, void* stream);

/* Best-epoch selection (nf_model/base.py:196-200) as device predicates:
 * *flag = (*a < *best), and *best = *a when true; fmc_copy_if copies
 * `bytes` from src to dst when *flag != 0. */
FMC_API int fmc_flag_less(const float* a, float* best, int32_t* flag, void* stream);
FMC_API int fmc_copy_if(const int32_t* flag, const void* src, void* dst, size_t bytes, void* stream);

/* data_mean and diag(data_cov) of x [n, d] (nf_model/base.py:187-188):
 * mean [d], unbiased variance [d]. Deterministic two-stage reduction whose
 * partials live in the caller's workspace (16-byte aligned, at least
 * fmc_column_stats_workspace_size bytes, at most 2 MiB). */
FMC_API int fmc_column_stats_workspace_size(int64_t n, int32_t d, size_t* bytes);
FMC_API int fmc_column_stats(const float* x, int64_t n, int32_t d, float* mean, float* var, void* ws,
                             size_t ws_bytes, void* stream);

/* dst[r] = src[perm(first + r)] for r < m, perm a pseudo-random permutation of
 * [0, n) keyed by (seed, counter): the epoch shuffle of NFModel.train_epoch
 * (nf_model/base.py:139-146). */
FMC_API int fmc_permute_rows(const float* src, int64_t n, int32_t d, uint64_t seed, uint64_t counter, int64_t first,
                             int64_t m, float* dst, void* stream);

/* TrainModel's data selection (strategy/train_model.py:66-80) from a chain
 * buffer buf [n_chains, n_steps, d]: rows with all-finite coordinates in
 * row-major order, reshaped to [n_chains, -1, d], the last history_window
 * rows of each, then n_out rows drawn with replacement (indices idx [n_out]
 * when non-NULL, else Philox(seed, counter)) -> out [n_out, d].
 * *err (device int32) is set to 1 when the finite rows do not split evenly
 * into n_chains (where the reference's reshape raises). */
FMC_API int fmc_select_workspace_size(int32_t n_chains, int64_t n_steps, size_t* bytes);
FMC_API int fmc_select_training_data(const float* buf, int32_t n_chains, int64_t n_steps, int32_t d,
                                     int32_t history_window, int64_t n_out, uint64_t seed, uint64_t counter,
                                     const int64_t* idx, float* out, int32_t* err, void* ws, size_t ws_bytes,
                                     void* stream);
/* The same selection without a workspace argument and without any device
 * allocation, for callers that cannot allocate device memory (code running
 * inside another framework's allocator or memory pool, or under a
 * no-allocation policy). No counterpart in the reference. Its scratch is a
 * static device array of about 12 MiB held by every GPU that loads the
 * library; it serves at most n_chains * n_steps = 1048576 rows and larger
 * buffers are rejected with FMC_ERR_INVALID_ARG. The first call on each
 * device looks the array's device address up (a synchronous runtime call), so
 * make that first call before any stream capture. All calls share the array:
 * calls that overlap on the GPU race, so serialise them. */
FMC_API int fmc_select_training_data_noalloc(const float* buf, int32_t n_chains, int64_t n_steps, int32_t d,
                                             int32_t history_window, int64_t n_out, uint64_t seed,
                                             uint64_t counter, const int64_t* idx, float* out, int32_t* err,
                                             void* stream);

/* ---- tensor-core GEMM (the conditioner's building block) ---------------- */
/* C = epilogue(A . B^T + bias) on tcgen05 with FP32 accumulation in TMEM.
 * A [rows_a, K] and B [rows_b, K] bf16 row-major (K a multiple of 64, rows_a
 * a multiple of 128 covering M, rows_b a multiple of 256 covering N).
 * epilogue 0: tanh -> bf16 C [M, ldc] (n_store columns, zeros beyond N);
 * epilogue 1: + bias -> fp32 C [M, ldc] (n_store = N columns). Replaces the
 * Linear + tanh layers of MLP.__call__ (resource/model/common.py:109-112). */
FMC_API int fmc_tc_gemm_bf16(const uint16_t* A, int64_t M, int64_t rows_a, int32_t K, const uint16_t* B,
                             int32_t N, int32_t rows_b, const float* bias, void* C, int64_t ldc, int32_t n_store,
                             int32_t epilogue, void* stream);
/* Failure-path self-test (no reference counterpart): runs the bounded
 * mbarrier wait of the tcgen05 kernels on a barrier that nothing completes.
 * *timed_out = 1 when the wait gave up (after about a second) and the kernel
 * returned normally; the context stays usable. Synchronises the stream. */
FMC_API int fmc_selftest_bounded_wait(int32_t* timed_out, void* stream);

/* Device error word of the tensor-core kernels: 1 after a bounded wait
 * expired (synchronous read; clear != 0 resets it). While the word is
 * raised, every later tensor-core launch returns at once without work (no
 * TMEM allocation, no waits), so a broken pipeline costs one wait bound in
 * total, not one per launch; the outputs of those launches are not written.
 * fmc_device_error_set writes the word (synchronous): clearing it after a
 * failure, or raising it to test the early return. */
FMC_API int fmc_device_error(int32_t* out, int32_t clear);
FMC_API int fmc_device_error_set(int32_t value);

/* ---- random streams under CUDA graph replay ------------------------- */
/* Attach a caller-owned device word (uint64) that every random stream of
 * the library folds into its key: launches made (or captured) after the
 * call read the word when they run, so a captured graph that advances it
 * draws fresh numbers on each replay. A zero word leaves the streams
 * unchanged; NULL detaches. Host-side setting, not thread-safe. */
FMC_API int fmc_rng_epoch_attach(uint64_t* word);
/* word += 1 on the stream (one tiny kernel; a graph node when captured). */
FMC_API int fmc_rng_epoch_advance(uint64_t* word, void* stream);

/* ---- library --------------------------------------------------------- */
FMC_API const char* fmc_last_error(void);
FMC_API int fmc_version(void);               /* FMC_ABI_VERSION */
/* Number of SMs of the current device (host call, synchronous). */
FMC_API int fmc_device_sm_count(int32_t* out);
/* Number of kernels this library has launched in the process (host counter). */
FMC_API int fmc_launch_count(uint64_t* out);

/* ---- streaming diagnostics (no counterpart in the reference, which
 * leaves diagnostics to arviz after sampling) -------------------------
 * FP64 accumulators of chain rows updated on the device while the sampler
 * runs: per chain and coordinate, Welford's running mean and sum of squared
 * deviations, and Welford over completed batch means of `batch` draws.
 * fmc_welford_ess_update folds rows [start, start + n_steps) of every chain
 * of a float32 buffer [n_chains, buf_len, n_dim] into the state (the draw
 * count is kept on the device, so a captured graph can replay updates).
 * fmc_welford_ess_finalize gives, per coordinate: the mean and the variance
 * of all draws, the multi-chain batch-means ESS (N var / (batch var_bm),
 * Flegal & Jones 2010; NaN with fewer than two completed batches) and
 * R-hat (Gelman & Rubin 1992). The state is caller-owned
 * (fmc_welford_state_size bytes, 8-byte aligned); fmc_welford_reset zeroes
 * it and sets the batch size. */
FMC_API int fmc_welford_state_size(int32_t n_chains, int32_t n_dim, size_t* bytes);
FMC_API int fmc_welford_reset(double* state, int32_t n_chains, int32_t n_dim, int32_t batch, void* stream);
FMC_API int fmc_welford_ess_update(const float* buf, int32_t n_chains, int64_t buf_len, int32_t n_dim,
                                   int64_t start, int32_t n_steps, double* state, void* stream);
FMC_API int fmc_welford_ess_finalize(const double* state, int32_t n_chains, int32_t n_dim, double* mean,
                                     double* var, double* ess, double* rhat, void* stream);

/* ---- per-kernel timing (profiling aid; no counterpart in the reference,
 * whose JAX path has no kernels of its own) ---------------------------
 * While enabled, every launch of the kernels listed below is bracketed by a
 * CUDA event pair recorded on its launch stream, and the launch's
 * algorithmic FLOPs and bytes (useful work, not padding) are noted. On a
 * stream that is capturing a CUDA graph the pair is recorded as external
 * event nodes of the graph: replay the graph before reading, and the times
 * are those of that replay, with the kernels back to back as the graph runs
 * them. fmc_kernel_timing_read synchronises on the recorded events and
 * returns the totals per kernel since the last reset; at most 16384 launches
 * are recorded between reads. Enabling creates the event pool on the
 * current device once. Off by default; costs two event records per timed
 * launch. */
enum {
  FMC_KT_TC_SPLINE_FWD = 0,   /* k_tc_spline, forward (fused last Linear + spline)  */
  FMC_KT_TC_SPLINE_INV = 1,   /* k_tc_spline, inverse                               */
  FMC_KT_TC_SPLINE_BWD = 2,   /* k_tc_spline_bwd (training adjoint)                 */
  FMC_KT_TC_GEMM_TANH = 3,    /* k_tc_gemm, bias + tanh -> bf16 (hidden layers)     */
  FMC_KT_TC_GEMM_DTANH = 4,   /* k_tc_gemm, tanh adjoint -> bf16 (backward)         */
  FMC_KT_TC_GEMM_F32 = 5,     /* k_tc_gemm, fp32 outputs (weight gradients)         */
  FMC_KT_LOCAL_STEPS = 6,     /* k_local_steps (MALA / HMC / GRW local phase)       */
  FMC_KT_NF_ACCEPT = 7,       /* k_nf_accept (target + independent-MH scan)         */
  FMC_KT_COUNT = 8
};
FMC_API int fmc_kernel_timing_enable(int32_t on);
FMC_API int fmc_kernel_timing_reset(void);
FMC_API int fmc_kernel_timing_read(int32_t kid, int64_t* launches, double* ms, double* flops, double* bytes);
/* Launch geometry of the last launch of kernel `kid` (whether or not timing
 * is on): CTAs in the grid and CTAs per cluster (2 for CTA pairs); 0, 0
 * before its first launch. */
FMC_API int fmc_kernel_grid(int32_t kid, int32_t* ctas, int32_t* cluster);

#ifdef __cplusplus
}
#endif
#endif /* FLOWMC_H */
