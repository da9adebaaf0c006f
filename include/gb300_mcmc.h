/*
 * gb300_mcmc.h -- C ABI of the GB300 (sm_103a) gradient-MCMC engine.
 *
 * Plain C: opaque handles, raw device pointers and sizes.  Every function
 * returns an int status (GBM_OK == 0); on failure gbm_last_error() returns a
 * thread-local message.  Numerical trouble (NaN/inf log-densities, divergent
 * trajectories) is never an error: it is reported in-band exactly as the
 * reference does (rejection, -inf log-accept ratios, divergence flags).
 *
 * Layouts: states are chain-major float32 [chains][dim] (the reference's
 * [C, D] batch layout, mcmc/hmc.py:184-192); log-densities, energies and
 * log-accept ratios are float64 [chains]; flags are uint8 [chains].
 * All tensor pointers are device pointers on the context's device; calls are
 * asynchronous on the context's stream unless stated otherwise.
 *
 * Reference paths are relative to tensorflow_probability/python/.
 */
#ifndef GB300_MCMC_H_
#define GB300_MCMC_H_

#include <stdint.h>

#if defined(__GNUC__)
#define GBM_API __attribute__((visibility("default")))
#else
#define GBM_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define GBM_OK 0
#define GBM_EINVAL 22
#define GBM_ENOMEM 12
#define GBM_ENOTSUP 95
#define GBM_ETIMEDOUT 110
#define GBM_ECUDA 1000

#define GBM_DTYPE_F32 0
#define GBM_DTYPE_BF16 1

/* Precision of a target's contractions.  F32: CUDA-core FP32 ("plain FP32").
 * MIXED: BF16 tensor-core contractions with FP32 accumulation and a
 * hi/lo split of the FP32 operands (residual correction). */
#define GBM_PRECISION_F32 0
#define GBM_PRECISION_MIXED 1

typedef struct gbm_context gbm_context;
typedef struct gbm_target gbm_target;
typedef struct gbm_hmc gbm_hmc;
typedef struct gbm_nuts gbm_nuts;

/* Library version (major * 10000 + minor * 100 + patch). */
GBM_API int gbm_version(void);

/* Message of the last failed call on this thread ("" if none). */
GBM_API const char* gbm_last_error(void);

/* Execution context: one device, one stream.  cuda_stream is the caller's
 * cudaStream_t (NULL = the device's default stream); every call of this
 * context is ordered on it.  There is no reference counterpart (TFP runs
 * on TensorFlow's device context, mcmc/nuts_test.py:516). */
GBM_API int gbm_context_create(int device, void* cuda_stream, gbm_context** out);
GBM_API int gbm_context_destroy(gbm_context* ctx);
GBM_API int gbm_context_synchronize(gbm_context* ctx);

/* Key of transition `step` in sample_chain's seed stream: the first two words
 * of Philox4x32-10(seed; step, STEP_KEY).  Replaces the reference's per-step
 * samplers.split_seed (mcmc/sample.py:344-349) with an addressable stream.
 * Host-only, no device work. */
GBM_API int gbm_step_key(const uint32_t seed[2], uint64_t step, uint32_t out[2]);

/* ---- target_log_prob_fn families ------------------------------------ */

/* Bayesian logistic regression: X [num_rows][num_features] (row-major,
 * dtype x_dtype), y [num_rows] float32 in {0,1}, iid Normal(0, prior_scale)
 * prior.  Replaces the user's target_log_prob_fn + autodiff
 * (mcmc/internal/util.py:286-308, math/gradient.py:28) for the
 * inference_gym logistic-regression target
 * (spinoffs/inference_gym/inference_gym/targets/logistic_regression.py:92-103,
 * distributions/bernoulli.py:126-140).  X and y are copied.  Kernels by
 * feature count: GBM_PRECISION_F32 (float32 X) runs fused CUDA-core kernels
 * up to 256 features; GBM_PRECISION_MIXED (float32 or BF16 X) fused tcgen05
 * kernels up to 512 (above 256 a 2-CTA cluster shares each tile).  Beyond
 * those limits the two contractions are cuBLAS GEMMs (FP32 accumulation; the
 * mixed form keeps the BF16 hi/lo residual correction) around this
 * library's element-wise kernels, and every evaluation covers all the
 * chains of the call.  num_rows < 2^31. */
GBM_API int gbm_target_logistic_regression(gbm_context* ctx, const void* x, int x_dtype,
                                   int64_t num_rows, int64_t num_features, const float* y,
                                   float prior_scale, int precision, gbm_target** out);
/* Multivariate normal MultivariateNormalTriL(loc, L) (distributions/
 * mvn_tril.py:44, mvn_linear_operator.py:242): loc [dim] and the inverse
 * scale factor L^-1 [dim][dim] (row-major, lower triangular, float32):
 * u = L^-1 (x - loc), logp = -1/2 |u|^2 + log_normalizer, grad = -L^-T u,
 * with log_normalizer = -sum log|L_ii| - dim/2 log 2pi supplied by the
 * caller. */
GBM_API int gbm_target_mvn(gbm_context* ctx, const float* loc, const float* scale_tril_inv,
                           int64_t dim, double log_normalizer, gbm_target** out);

/* Non-centred hierarchical normal (the eight-schools model of
 * mcmc/eight_schools_hmc.py:41-58): mu ~ N(0, mu_scale), tau ~
 * HalfCauchy(0, tau_scale), z_j ~ N(0, 1), y_j ~ N(mu + tau z_j, sigma_j),
 * j < groups.  State [mu, log tau, z_1..z_groups] (dim = groups + 2); the
 * log-density includes the log-Jacobian of tau = exp(log tau), as
 * TransformedTransitionKernel with an Exp bijector gives
 * (mcmc/transformed_kernel.py:165).  y, sigma: float32 [groups]. */
GBM_API int gbm_target_hierarchical_normal(gbm_context* ctx, const float* y, const float* sigma,
                                           int64_t groups, float mu_scale, float tau_scale,
                                           gbm_target** out);

/* Many independent posteriors of uneven dimension in one target, for one
 * NoUTurnSampler over all of them (one set of launches per sampler step for
 * every member).  Each member is a multivariate normal (loc, L^-1 and
 * log_normalizer as for gbm_target_mvn) or a non-centred hierarchical normal
 * (group_y, group_sigma, mu_scale, tau_scale as for
 * gbm_target_hierarchical_normal; its state dimension is dim + 2), with its
 * own number of chains.  There is no single reference object for this: it
 * replaces running one tfp.mcmc.NoUTurnSampler (mcmc/nuts.py:165) per
 * posterior with per-chain step sizes (nuts.py:237-243 allows [C, 1] step
 * sizes).  States, gradients and momenta are ragged: member t's chains come
 * after member t-1's, and chain c's vector has dims[c] float32 elements
 * starting at element offsets[c] (gbm_target_batch_layout).  The
 * log-density of every chain is one float64.  Inputs are copied. */
typedef struct gbm_batch_member {
  int32_t family;                 /* GBM_FAMILY_MVN or GBM_FAMILY_HIERARCHICAL_NORMAL */
  int64_t dim;                    /* MVN: state dimension; hierarchical: groups J */
  int64_t chains;                 /* chains sampling this posterior */
  const float* loc;               /* MVN [dim] */
  const float* scale_tril_inv;    /* MVN [dim][dim], lower triangular */
  double log_normalizer;          /* MVN */
  const float* group_y;           /* hierarchical [J] */
  const float* group_sigma;       /* hierarchical [J] */
  float mu_scale, tau_scale;      /* hierarchical */
} gbm_batch_member;

GBM_API int gbm_target_batch(gbm_context* ctx, const gbm_batch_member* members, int64_t count,
                             gbm_target** out);
/* Ragged layout of a batch target (host arrays of `chains` entries, either
 * may be NULL): per-chain element offsets and dimensions, the number of
 * chains and the total number of state elements. */
GBM_API int gbm_target_batch_layout(const gbm_target* target, int64_t* offsets, int32_t* dims,
                                    int64_t* chains, int64_t* elements);
/* Chain-tile width (32 or 64 chains) the construction-time autotuner chose
 * for multivariate-normal members with dim <= 64, <= 256, <= 1024 and
 * > 1024 (0: no member in that class). */
GBM_API int gbm_target_batch_schedule(const gbm_target* target, int32_t chain_tile[4]);

/* The target `inner` seen through one elementwise bijector per state
 * dimension, for TransformedTransitionKernel (mcmc/transformed_kernel.py:165;
 * the transformed log-density of make_transformed_log_prob,
 * transformed_kernel.py:63-95): states x are unconstrained, `inner` is
 * evaluated at y = f(x), and log |f'(x)| (float64) is added with the chain
 * rule applied to the gradient.  bijector[d] is GBM_BIJECTOR_* (the forward
 * maps of bijectors/exp.py, softplus.py, sigmoid.py).  `inner` must outlive
 * the returned target and must not be a batch target. */
#define GBM_BIJECTOR_IDENTITY 0
#define GBM_BIJECTOR_EXP 1
#define GBM_BIJECTOR_SOFTPLUS 2
#define GBM_BIJECTOR_SIGMOID 3
GBM_API int gbm_target_transformed(gbm_target* inner, const int32_t* bijector, gbm_target** out);

GBM_API int gbm_target_destroy(gbm_target* target);
GBM_API int gbm_target_dim(const gbm_target* target, int64_t* dim);

/* Batched log-density and gradient at `chains` states (the value-and-gradient
 * call of mcmc/internal/util.py:246-283).  log_prob: float64 [chains];
 * grad: float32 [chains][dim].  Asynchronous on the context stream; a
 * bounded device wait that timed out in an earlier call is reported here
 * (GBM_ETIMEDOUT) or by gbm_context_synchronize. */
GBM_API int gbm_target_log_prob_and_grad(gbm_target* target, const float* state, int64_t chains,
                                 double* log_prob, float* grad);

/* Allocation-free logistic-regression log-density and gradient.  No
 * counterpart in the reference: it serves callers that cannot allocate
 * device memory -- framework custom-call/custom-op slots that hand in only
 * their own input and output buffers, and serving loops that must not
 * synchronise the device through cudaMalloc/cudaFree.  Same results as
 * gbm_target_log_prob_and_grad on a GBM_PRECISION_F32 target, but X [N][D]
 * float32 and y [N] are the caller's device buffers (no copy, no handle) and
 * the scratch is a fixed 8 MiB device array inside this library, held on
 * every GPU that loads it until the process exits.  Runs on the current
 * device, asynchronously on cuda_stream (NULL = default stream).
 * Limits: 1 <= num_features <= 256; chains <= 64 * min(2 * SMs,
 * floor((8 MiB - 256) / (64 * (8 + 4 * num_features)))) -- 19456 chains at
 * 100 features on GB300; larger requests fail with GBM_EINVAL.  The first
 * call on a device resolves the scratch array's device address
 * (cudaGetSymbolAddress) and sets kernel attributes; make that first call
 * before any stream capture.  Calls share the one scratch array: calls that
 * overlap on the GPU (other streams, other host threads) race and must be
 * serialised by the caller.  Allocates nothing. */
GBM_API int gbm_logreg_log_prob_and_grad_noalloc(const float* x, int64_t num_rows,
                                                 int64_t num_features, const float* y,
                                                 float prior_scale, const float* state,
                                                 int64_t chains, double* log_prob, float* grad,
                                                 void* cuda_stream);

/* Algorithmic flops and HBM bytes of one batched evaluation at `chains`. */
GBM_API int gbm_target_cost(const gbm_target* target, int64_t chains, double* flops, double* bytes);

/* ---- HamiltonianMonteCarlo ------------------------------------------- */

/* One transition of MetropolisHastings(UncalibratedHamiltonianMonteCarlo)
 * (mcmc/hmc.py:501-529 -> mcmc/metropolis_hastings.py:160-254,
 * mcmc/hmc.py:661-729).  step_size: float32 device scalar, or [chains] when
 * step_size_per_chain != 0.  seed: 2 x uint32 host words keying the
 * momentum and MH-uniform draws.  Any of the optional outputs
 * (proposed_*, initial_momentum, final_momentum, log_acceptance_correction)
 * may be NULL. */
GBM_API int gbm_hmc_create(gbm_target* target, int64_t max_chains, gbm_hmc** out);
GBM_API int gbm_hmc_destroy(gbm_hmc* kernel);
GBM_API int gbm_hmc_one_step(gbm_hmc* kernel, int64_t chains, const float* state,
                     const double* target_log_prob, const float* grads_target_log_prob,
                     const float* step_size, int step_size_per_chain,
                     int32_t num_leapfrog_steps, const uint32_t seed[2],
                     float* next_state, double* next_target_log_prob,
                     float* next_grads_target_log_prob, float* proposed_state,
                     double* proposed_target_log_prob, float* proposed_grads_target_log_prob,
                     float* initial_momentum, float* final_momentum,
                     double* log_acceptance_correction, double* log_accept_ratio,
                     uint8_t* is_accepted);

/* ---- NoUTurnSampler -------------------------------------------------- */

/* NoUTurnSampler(target, step_size, max_tree_depth, max_energy_diff,
 * unrolled_leapfrog_steps) (mcmc/nuts.py:197-275).  Allocates the
 * per-chain trajectory workspace for up to max_chains chains. */
GBM_API int gbm_nuts_create(gbm_target* target, int64_t max_chains, int32_t max_tree_depth,
                    double max_energy_diff, int32_t unrolled_leapfrog_steps, gbm_nuts** out);
GBM_API int gbm_nuts_destroy(gbm_nuts* kernel);

/* NoUTurnSampler.one_step (mcmc/nuts.py:321-445).  Outputs are the fields of
 * NUTSKernelResults (nuts.py:74-91) plus the next state; tree_depth may be
 * NULL.  Blocks the host at most once per tree depth to read whether any
 * chain continues (the reference's tf.while_loop condition, nuts.py:404-407). */
GBM_API int gbm_nuts_one_step(gbm_nuts* kernel, int64_t chains, const float* state,
                      const double* target_log_prob, const float* grads_target_log_prob,
                      const float* step_size, int step_size_per_chain, const uint32_t seed[2],
                      float* next_state, double* next_target_log_prob,
                      float* next_grads_target_log_prob, double* log_accept_ratio,
                      int32_t* leapfrogs_taken, uint8_t* is_accepted, uint8_t* reach_max_depth,
                      uint8_t* has_divergence, double* energy, int32_t* tree_depth);

/* Free-running NoUTurnSampler transitions.  No single reference call: each
 * chain runs `transitions_per_chain` transitions of NoUTurnSampler.one_step
 * (mcmc/nuts.py:321-445) with keys gbm_step_key(seed, first_step + t) -- the
 * transitions sample_chain (mcmc/sample.py:81-383) would run at a fixed step
 * size -- but not in lock-step: a chain starts its next transition as soon as
 * its own trajectory ends, so one chain building a depth-10 tree does not
 * hold every other chain for 1023 leaves.  Per chain the results equal the
 * lock-step sampler's with the same keys.  One leaf iteration advances every
 * running chain by one leapfrog step; the run stops when every chain has
 * finished or after max_leaf_iterations (chains are then left mid-way and
 * transitions_done says how many each completed).  Inputs as
 * gbm_nuts_one_step (step_size [1] or [chains]); unrolled_leapfrog_steps
 * must be 1.  Device outputs, each may be NULL: transitions_done int32
 * [chains]; trace [transitions_per_chain][...] of the completed transitions:
 * states (float32, [state elements] each), target log-probs, log-accept
 * ratios (float64 [chains]), leapfrogs taken (int32), accepted and
 * divergence flags (uint8).  leaf_iterations (host, may be NULL): the
 * iterations run. */
GBM_API int gbm_nuts_run_free(gbm_nuts* kernel, int64_t chains, const float* state,
                              const double* target_log_prob, const float* grads_target_log_prob,
                              const float* step_size, int step_size_per_chain,
                              const uint32_t seed[2], int64_t first_step,
                              int32_t transitions_per_chain, int64_t max_leaf_iterations,
                              int32_t* transitions_done, float* trace_state,
                              double* trace_target_log_prob, double* trace_log_accept_ratio,
                              int32_t* trace_leapfrogs_taken, uint8_t* trace_is_accepted,
                              uint8_t* trace_has_divergence, int64_t* leaf_iterations);

/* Number of leaf iterations (batched gradient evaluations) the last
 * gbm_nuts_one_step (or gbm_nuts_run_free) launched. */
GBM_API int gbm_nuts_last_leaf_iterations(const gbm_nuts* kernel, int64_t* out);

/* Profiling of NUTS transitions.  When enabled, CUDA events on the context
 * stream bracket every batched target evaluation.  gbm_nuts_read_profile
 * synchronizes the stream and returns, since the previous read, the summed
 * device time of those evaluations (ms), their count, and the number of
 * kernels this handle launched (targets' kernels included), then resets. */
GBM_API int gbm_nuts_set_profiling(gbm_nuts* kernel, int enable);
/* CUDA-graph replay of the per-leaf launch sequence (on by default; steps
 * taken while profiling is on always launch leaf by leaf).  Replay gives the
 * same bits as per-leaf launches.  No reference counterpart: tfp.mcmc runs
 * under tf.function/XLA, which this replaces. */
GBM_API int gbm_nuts_set_graphs(gbm_nuts* kernel, int enable);
/* Free-running draws in gbm_nuts_sample_chain (off by default): the results
 * whose transitions all run at the final step size (dual averaging past its
 * window, or no adaptation) and no thinning come from the free-running loop
 * of gbm_nuts_run_free -- per chain the same transitions (keys, step size,
 * trace rows, streaming moments, final state), but no chain waits for the
 * batch's longest trajectory.  The dual-averaging state then advances with
 * every transition's accept ratio in order, as in lock-step.  For targets
 * whose per-chain arithmetic does not depend on which chains are evaluated
 * together (the multivariate-normal and hierarchical families) the results
 * are bit-equal to lock-step; the logistic-regression kernels' row splits
 * depend on the active-chain count, so there they agree to rounding.  No
 * reference counterpart (tfp.mcmc runs every chain in lock-step). */
GBM_API int gbm_nuts_set_free_running(gbm_nuts* kernel, int enable);
/* Streaming moments on the device (for the running potential scale
 * reduction of experimental/mcmc/potential_scale_reduction_reducer.py and
 * diagnostic.py:476-568 without storing draws): fold one state of
 * `elements` float32 values into per-element running means and sums of
 * squared deviations (float64, Welford) after `count_before` samples. */
GBM_API int gbm_moments_update(gbm_context* ctx, const float* state, int64_t elements,
                               int64_t count_before, double* mean, double* m2);
/* Streaming autocovariance for the effective sample size
 * (mcmc/diagnostic.py:203-337 with filter_beyond_lag = max_lag) without
 * storing draws: fold one state of `elements` float32 values, the
 * (count_before + 1)-th draw, into per-element running sums.  With E =
 * elements and L = max_lag, the caller's zero-initialised device arrays are
 * first [E] and head, ring [L][E] (float32), total [E] and lag_sums [L+1][E]
 * (float64): first holds x_0, head the first L and ring the last L draws
 * (ring[t mod L]); with y_t = x_t - x_0 in float64, total = sum y_t and
 * lag_sums[k] = sum_{t >= k} y_t y_{t-k} -- from which the centred
 * autocovariance at lags 0..L follows exactly. */
GBM_API int gbm_autocov_update(gbm_context* ctx, const float* state, int64_t elements,
                               int64_t count_before, int32_t max_lag, float* first,
                               double* total, float* head, float* ring, double* lag_sums);
/* Diagonal mass matrix for subsequent gbm_nuts_one_step calls, as
 * tfp.experimental.mcmc.PreconditionedNoUTurnSampler
 * (experimental/mcmc/preconditioned_nuts.py:169) with the momentum
 * distribution DiagonalMassMatrixAdaptation builds
 * (experimental/mcmc/preconditioning_utils.py:40-97): precision diag(v),
 * i.e. momentum p ~ N(0, diag(1/v)), velocity v * p, kinetic energy
 * 1/2 sum v p^2, U-turn checks against velocities.  `inverse_mass` is v, a
 * device pointer read by every later step (keep it alive; it may be
 * updated in place): float32 [dim] shared by all chains, or with per_chain
 * one value per state element.  NULL restores the identity (the
 * NoUTurnSampler of nuts.py).  The energy reported excludes the momentum
 * distribution's normalizer. */
GBM_API int gbm_nuts_set_inverse_mass(gbm_nuts* kernel, const float* inverse_mass,
                                      int per_chain);
GBM_API int gbm_nuts_read_profile(gbm_nuts* kernel, double* eval_ms, int64_t* evals,
                                  int64_t* kernel_launches);

/* ---- sample_chain ------------------------------------------------------- */

/* sample_chain (mcmc/sample.py:81-383) over NoUTurnSampler, optionally inside
 * DualAveragingStepSizeAdaptation, run entirely on the device: result 0
 * after 1 + num_burnin_steps transitions, then one result every
 * 1 + num_steps_between_results.  Transition t uses gbm_step_key(seed,
 * first_step + t).  state/target_log_prob/grads (in: current, out: final)
 * and step_size (float32 [1] or [chains]; in: next step size, out: final)
 * are updated in place.  num_adaptation_steps <= 0 disables adaptation;
 * otherwise da_state is the float64 [groups][4] dual-averaging state of
 * gbm_dual_averaging_update (in/out).  Trace pointers ([num_results][...],
 * device) may each be NULL.  Blocks the host at most once per tree depth
 * per transition. */
GBM_API int gbm_nuts_sample_chain(gbm_nuts* kernel, int64_t chains, float* state,
                                  double* target_log_prob, float* grads_target_log_prob,
                                  float* step_size, int step_size_per_chain,
                                  const uint32_t seed[2], int64_t first_step,
                                  int64_t num_results, int64_t num_burnin_steps,
                                  int64_t num_steps_between_results,
                                  int32_t num_adaptation_steps, double target_accept_prob,
                                  double exploration_shrinkage, double step_count_smoothing,
                                  double decay_rate, double* da_state, float* trace_state,
                                  double* trace_target_log_prob, double* trace_log_accept_ratio,
                                  int32_t* trace_leapfrogs_taken, uint8_t* trace_is_accepted,
                                  uint8_t* trace_has_divergence, float* trace_step_size);

/* The same loop over MetropolisHastings(UncalibratedHamiltonianMonteCarlo)
 * with num_leapfrog_steps leapfrog steps per transition; fully asynchronous. */
GBM_API int gbm_hmc_sample_chain(gbm_hmc* kernel, int64_t chains, float* state,
                                 double* target_log_prob, float* grads_target_log_prob,
                                 float* step_size, int step_size_per_chain,
                                 int32_t num_leapfrog_steps, const uint32_t seed[2],
                                 int64_t first_step, int64_t num_results,
                                 int64_t num_burnin_steps, int64_t num_steps_between_results,
                                 int32_t num_adaptation_steps, double target_accept_prob,
                                 double exploration_shrinkage, double step_count_smoothing,
                                 double decay_rate, double* da_state, float* trace_state,
                                 double* trace_target_log_prob, double* trace_log_accept_ratio,
                                 uint8_t* trace_is_accepted, float* trace_step_size);

/* ---- Job server: many independent posteriors at once ------------------- */

/* There is no counterpart in the reference (it runs one sample_chain per
 * Python call).  A server owns `workers` host threads, each with two device
 * streams (the device's greatest and least priority; jobs with little work
 * per leaf run on the first).  Jobs -- one target family + DA(NUTS)
 * sample_chain run, the draws past the adaptation window free-running as
 * with gbm_nuts_set_free_running -- are admitted first-in first-out while
 * their estimated device memory fits `memory_budget_bytes`; admitted jobs
 * run concurrently on the workers' streams with all chain and adaptation
 * state resident on the device, and their buffers come from the
 * stream-ordered allocator so job set-up and tear-down never synchronize
 * the device.  Kernels are deterministic, so a job's results do not depend
 * on what else runs beside it. */
#define GBM_FAMILY_LOGISTIC_REGRESSION 0
#define GBM_FAMILY_MVN 1
#define GBM_FAMILY_HIERARCHICAL_NORMAL 2

#define GBM_JOB_QUEUED 0
#define GBM_JOB_RUNNING 1
#define GBM_JOB_DONE 2
#define GBM_JOB_FAILED 3

typedef struct gbm_server gbm_server;

/* One posterior-sampling job.  Input pointers are device pointers that must
 * stay valid until the job is DONE or FAILED; output pointers may be NULL. */
typedef struct gbm_job_spec {
  int32_t family;                 /* GBM_FAMILY_* */
  /* logistic regression: x [rows][features] (x_dtype), y [rows] */
  const void* x;
  int32_t x_dtype;
  int32_t precision;              /* GBM_PRECISION_* */
  int64_t rows;
  int64_t features;
  const float* y;
  float prior_scale;
  /* multivariate normal: loc [dim], scale_tril_inv [dim][dim] */
  const float* loc;
  const float* scale_tril_inv;
  double log_normalizer;
  /* hierarchical normal: group_y, group_sigma [groups] */
  const float* group_y;
  const float* group_sigma;
  int64_t groups;
  float mu_scale;
  float tau_scale;
  /* sampler: DualAveragingStepSizeAdaptation(NoUTurnSampler) */
  int64_t dim;                    /* must match the family's dimension */
  int64_t chains;
  const float* init_state;        /* [chains][dim] */
  float step_size;                /* initial step size */
  int32_t max_tree_depth;
  int32_t num_adaptation_steps;   /* <= 0: fixed step size */
  double target_accept_prob;
  int64_t num_results;
  int64_t num_burnin_steps;
  uint32_t seed[2];
  /* outputs (device) */
  float* trace_state;             /* [num_results][chains][dim] */
  double* trace_log_accept_ratio; /* [num_results][chains] */
  int32_t* trace_leapfrogs_taken; /* [num_results][chains] */
  float* final_state;             /* [chains][dim] */
  float* final_step_size;         /* [1] */
  /* optional streaming moments of the draws (float64 [chains][dim] each):
   * per-chain mean and sum of squared deviations, for R-hat without the
   * trace (gbm_moments_update) */
  double* moments_mean;
  double* moments_m2;
} gbm_job_spec;

typedef struct gbm_job_info {
  int32_t status;                 /* GBM_JOB_* */
  int32_t error_code;             /* GBM_* status of a failed job */
  double submit_s, start_s, end_s;  /* server clock (s since creation) */
  int64_t device_bytes;           /* admission estimate */
} gbm_job_info;

GBM_API int gbm_server_create(int device, int32_t workers, int64_t memory_budget_bytes,
                              gbm_server** out);
/* Waits for running jobs to finish and drops queued ones. */
GBM_API int gbm_server_destroy(gbm_server* server);
GBM_API int gbm_server_submit(gbm_server* server, const gbm_job_spec* spec, int64_t* job_id);
GBM_API int gbm_server_query(gbm_server* server, int64_t job_id, gbm_job_info* info);
/* Blocks until the job is DONE or FAILED or `timeout_s` passes
 * (GBM_ETIMEDOUT). */
GBM_API int gbm_server_wait(gbm_server* server, int64_t job_id, double timeout_s,
                            gbm_job_info* info);
/* Forget a finished job's record. */
GBM_API int gbm_server_release(gbm_server* server, int64_t job_id);
/* Seconds since the server was created (the clock of gbm_job_info). */
GBM_API double gbm_server_now(gbm_server* server);

/* ---- DualAveragingStepSizeAdaptation ----------------------------------- */

/* One dual-averaging update after an inner one_step
 * (mcmc/dual_averaging_step_size_adaptation.py:353-475, 477-532).
 * log_accept_ratio: float64 [chains] from the inner kernel.
 * state: float64 [groups][4] = (error_sum, log_averaging_step,
 * log_shrinkage_target, step) with groups = 1 (shared step size, chains
 * reduced by reduce_logmeanexp) or chains (per-chain step sizes).
 * step_size: float32 [groups]; on entry the step size used by this
 * transition, on exit the next one (new_step_size).  target_accept_prob:
 * float64 [groups] device array, or NULL to use `target_accept_scalar`. */
GBM_API int gbm_dual_averaging_update(gbm_context* ctx, int64_t chains, const double* log_accept_ratio,
                              int per_chain, int32_t num_adaptation_steps,
                              double target_accept_scalar, const double* target_accept_prob,
                              double exploration_shrinkage, double step_count_smoothing,
                              double decay_rate, double* state, float* step_size);

/* The same update with the chains' log accept probabilities already reduced
 * by the caller: reduced_log_accept_prob is float64 [groups], the value of
 * DualAveragingStepSizeAdaptation's reduce_fn (reduce_logmeanexp by default;
 * e.g. reduce_log_harmonic_mean_exp or a maximum, as the reference allows,
 * dual_averaging_step_size_adaptation.py:141,410-422) applied to
 * min(log_accept_ratio, 0) (non-finite -> -inf). */
GBM_API int gbm_dual_averaging_update_reduced(gbm_context* ctx, int64_t groups,
                                              const double* reduced_log_accept_prob,
                                              int32_t num_adaptation_steps,
                                              double target_accept_scalar,
                                              const double* target_accept_prob,
                                              double exploration_shrinkage,
                                              double step_count_smoothing, double decay_rate,
                                              double* state, float* step_size);

/* ---- MetropolisHastings ----------------------------------------------- */

/* MetropolisHastings.one_step's accept/reject for a proposal an inner kernel
 * already made (mcmc/metropolis_hastings.py:160-254): log_accept_ratio =
 * proposed - current target log-prob + log_acceptance_correction (NULL: 0),
 * non-finite -> -inf (safe_sum, mcmc/internal/util.py:213-235); accept iff
 * log U < log_accept_ratio with U the transition's Metropolis-Hastings
 * uniform for `seed` (the draw gbm_hmc_one_step uses, so wrapping the
 * uncalibrated HMC proposal reproduces gbm_hmc_one_step exactly);
 * next_state = accepted ? proposed : current ([chains][dim] float32). */
GBM_API int gbm_metropolis_hastings_step(gbm_context* ctx, int64_t chains, int64_t dim,
                                         const uint32_t seed[2],
                                         const double* current_target_log_prob,
                                         const double* proposed_target_log_prob,
                                         const double* log_acceptance_correction,
                                         const float* current_state, const float* proposed_state,
                                         float* next_state, double* log_accept_ratio,
                                         uint8_t* is_accepted);

#ifdef __cplusplus
}
#endif

#endif  /* GB300_MCMC_H_ */
