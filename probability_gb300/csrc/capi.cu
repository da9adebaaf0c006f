// C-ABI entry points (include/gb300_mcmc.h): argument checks, error
// reporting, handle lifetime.  All numerical work is in the kernels of
// logreg_*.cu and samplers.cu.
#include <cuda_runtime.h>

#include <cstdio>
#include <new>
#include <string>

#include "gb300_mcmc.h"
#include "rng.cuh"
#include "samplers.h"

namespace gbm {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }

void context_init(gbm_context* ctx, int device, cudaStream_t stream, bool owns_stream) {
  ctx->device = device;
  ctx->stream = stream;   // NULL: the default stream
  ctx->owns_stream = owns_stream;
  GBM_CUDA(cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device));
  ctx->host_flag_slots = 16;
  GBM_CUDA(cudaMallocHost(&ctx->host_flags, sizeof(int) * ctx->host_flag_slots));
  void* errp = nullptr;
  GBM_CUDA(cudaHostAlloc(&errp, 64, cudaHostAllocMapped));
  ctx->err_host = static_cast<volatile int*>(errp);
  *ctx->err_host = 0;
  GBM_CUDA(cudaHostGetDevicePointer(reinterpret_cast<void**>(&ctx->err_dev), errp, 0));
}

void context_free(gbm_context* ctx) {
  cudaStreamSynchronize(ctx->stream);
  if (ctx->host_flags) cudaFreeHost(ctx->host_flags);
  if (ctx->err_host) cudaFreeHost(const_cast<int*>(ctx->err_host));
  if (ctx->owns_stream) cudaStreamDestroy(ctx->stream);
  ctx->host_flags = nullptr;
  ctx->err_host = nullptr;
}

std::unique_ptr<Target> make_logreg_tc(gbm_context* ctx, const void* X, int x_dtype, int64_t n,
                                       int64_t d, const float* y, float prior_scale);

}  // namespace gbm

using gbm::set_error;

namespace {

template <class F>
int guarded(F&& f) {
  try {
    return f();
  } catch (const gbm::CudaError& e) {
    set_error(std::string(e.what) + ": " + cudaGetErrorString(e.err));
    return e.err == cudaErrorMemoryAllocation ? GBM_ENOMEM : GBM_ECUDA;
  } catch (const gbm::DeviceTimeout& e) {
    set_error("a bounded device wait timed out inside a kernel (code " +
              std::to_string(e.code) + ")");
    return GBM_ETIMEDOUT;
  } catch (const std::bad_alloc&) {
    set_error("host allocation failed");
    return GBM_ENOMEM;
  } catch (const std::exception& e) {
    set_error(e.what());
    return GBM_EINVAL;
  }
}

int invalid(const std::string& msg) {
  set_error(msg);
  return GBM_EINVAL;
}

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    int cur = -1;
    cudaGetDevice(&cur);
    if (prev >= 0 && cur != prev) cudaSetDevice(prev);
  }
};

}  // namespace

extern "C" {

int gbm_version(void) { return 100; }

const char* gbm_last_error(void) { return gbm::g_last_error.c_str(); }

int gbm_step_key(const uint32_t seed[2], uint64_t step, uint32_t out[2]) {
  if (!seed || !out) return invalid("gbm_step_key: NULL argument");
  if (step >= ((uint64_t)1 << 32)) return invalid("gbm_step_key: step must be < 2^32");
  const uint2 k = gbm::step_key(make_uint2(seed[0], seed[1]), (uint32_t)step);
  out[0] = k.x;
  out[1] = k.y;
  return GBM_OK;
}

int gbm_context_create(int device, void* stream, gbm_context** out) {
  if (!out) return invalid("gbm_context_create: out is NULL");
  return guarded([&] {
    int n = 0;
    GBM_CUDA(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n) return invalid("gbm_context_create: bad device index");
    DeviceGuard g(device);
    auto* ctx = new gbm_context();
    gbm::context_init(ctx, device, static_cast<cudaStream_t>(stream), false);
    *out = ctx;
    return GBM_OK;
  });
}

int gbm_context_destroy(gbm_context* ctx) {
  if (!ctx) return GBM_OK;
  return guarded([&] {
    DeviceGuard g(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    if (ctx->host_flags) cudaFreeHost(ctx->host_flags);
    if (ctx->err_host) cudaFreeHost(const_cast<int*>(ctx->err_host));
    if (ctx->owns_stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return GBM_OK;
  });
}

int gbm_context_synchronize(gbm_context* ctx) {
  if (!ctx) return invalid("gbm_context_synchronize: ctx is NULL");
  return guarded([&] {
    DeviceGuard g(ctx->device);
    GBM_CUDA(cudaStreamSynchronize(ctx->stream));
    gbm::check_device_error(ctx);
    return GBM_OK;
  });
}

int gbm_target_logistic_regression(gbm_context* ctx, const void* x, int x_dtype,
                                   int64_t num_rows, int64_t num_features, const float* y,
                                   float prior_scale, int precision, gbm_target** out) {
  if (!ctx || !x || !y || !out) return invalid("gbm_target_logistic_regression: NULL argument");
  if (num_rows <= 0 || num_features <= 0)
    return invalid("gbm_target_logistic_regression: num_rows and num_features must be > 0");
  if (num_rows > (int64_t)1 << 31)
    return invalid("gbm_target_logistic_regression: num_rows must be < 2^31");
  if (!(prior_scale > 0.f))
    return invalid("gbm_target_logistic_regression: prior_scale must be > 0");
  if (x_dtype != GBM_DTYPE_F32 && x_dtype != GBM_DTYPE_BF16)
    return invalid("gbm_target_logistic_regression: x_dtype must be GBM_DTYPE_F32 or BF16");
  if (precision != GBM_PRECISION_F32 && precision != GBM_PRECISION_MIXED)
    return invalid("gbm_target_logistic_regression: unknown precision");
  return guarded([&] {
    DeviceGuard g(ctx->device);
    auto* t = new gbm_target();
    t->ctx = ctx;
    if (precision == GBM_PRECISION_F32) {
      if (x_dtype != GBM_DTYPE_F32) {
        delete t;
        return invalid("gbm_target_logistic_regression: FP32 precision needs float32 X");
      }
      t->impl = gbm::make_logreg_simt(ctx, static_cast<const float*>(x), num_rows, num_features,
                                      y, prior_scale);
      if (!t->impl)   // above 256 features: library GEMMs + fused element-wise kernels
        t->impl = gbm::make_logreg_large(ctx, x, x_dtype, num_rows, num_features, y,
                                         prior_scale, false);
      if (!t->impl) {
        delete t;
        return invalid("gbm_target_logistic_regression: shape out of range");
      }
    } else {
      t->impl = gbm::make_logreg_tc(ctx, x, x_dtype, num_rows, num_features, y, prior_scale);
      if (!t->impl)   // above 512 features
        t->impl = gbm::make_logreg_large(ctx, x, x_dtype, num_rows, num_features, y,
                                         prior_scale, true);
      if (!t->impl) {
        delete t;
        set_error("gbm_target_logistic_regression: mixed-precision path unavailable for this shape");
        return GBM_ENOTSUP;
      }
    }
    GBM_CUDA(cudaMalloc(&t->count.ptr, sizeof(int)));
    t->count.bytes = sizeof(int);
    GBM_CUDA(cudaStreamSynchronize(ctx->stream));
    *out = t;
    return GBM_OK;
  });
}

static int finish_target(gbm_context* ctx, gbm_target* t, gbm_target** out) {
  GBM_CUDA(cudaMalloc(&t->count.ptr, sizeof(int)));
  t->count.bytes = sizeof(int);
  GBM_CUDA(cudaStreamSynchronize(ctx->stream));
  *out = t;
  return GBM_OK;
}

int gbm_target_mvn(gbm_context* ctx, const float* loc, const float* precision, int64_t dim,
                   double log_normalizer, gbm_target** out) {
  if (!ctx || !loc || !precision || !out) return invalid("gbm_target_mvn: NULL argument");
  if (dim <= 0 || dim > 65536) return invalid("gbm_target_mvn: dim must be in [1, 65536]");
  return guarded([&] {
    DeviceGuard g(ctx->device);
    std::unique_ptr<gbm_target> t(new gbm_target());
    t->ctx = ctx;
    t->impl = gbm::make_mvn(ctx, loc, precision, dim, log_normalizer);
    finish_target(ctx, t.get(), out);
    t.release();
    return GBM_OK;
  });
}

int gbm_target_hierarchical_normal(gbm_context* ctx, const float* y, const float* sigma,
                                   int64_t groups, float mu_scale, float tau_scale,
                                   gbm_target** out) {
  if (!ctx || !y || !sigma || !out) return invalid("gbm_target_hierarchical_normal: NULL argument");
  if (groups <= 0 || groups > (1 << 24)) return invalid("gbm_target_hierarchical_normal: bad groups");
  if (!(mu_scale > 0.f) || !(tau_scale > 0.f))
    return invalid("gbm_target_hierarchical_normal: scales must be > 0");
  return guarded([&] {
    DeviceGuard g(ctx->device);
    std::unique_ptr<gbm_target> t(new gbm_target());
    t->ctx = ctx;
    t->impl = gbm::make_hier(ctx, y, sigma, groups, mu_scale, tau_scale);
    finish_target(ctx, t.get(), out);
    t.release();
    return GBM_OK;
  });
}

int gbm_target_batch(gbm_context* ctx, const gbm_batch_member* m, int64_t count,
                     gbm_target** out) {
  if (!ctx || !m || !out) return invalid("gbm_target_batch: NULL argument");
  if (count <= 0 || count > (1 << 20)) return invalid("gbm_target_batch: bad member count");
  int64_t chains = 0, elems = 0;
  for (int64_t i = 0; i < count; ++i) {
    const gbm_batch_member& b = m[i];
    if (b.chains <= 0 || b.dim <= 0 || b.dim > (1 << 16))
      return invalid("gbm_target_batch: every member needs chains > 0 and 0 < dim <= 65536");
    if (b.family == GBM_FAMILY_MVN) {
      if (!b.loc || !b.scale_tril_inv) return invalid("gbm_target_batch: MVN member needs loc, L^-1");
    } else if (b.family == GBM_FAMILY_HIERARCHICAL_NORMAL) {
      if (!b.group_y || !b.group_sigma || !(b.mu_scale > 0.f) || !(b.tau_scale > 0.f))
        return invalid("gbm_target_batch: hierarchical member needs y, sigma and scales > 0");
    } else {
      return invalid("gbm_target_batch: members are MVN or hierarchical-normal");
    }
    chains += b.chains;
    elems += b.chains * (b.family == GBM_FAMILY_MVN ? b.dim : b.dim + 2);
  }
  if (chains > (1 << 24) || elems > ((int64_t)1 << 34))
    return invalid("gbm_target_batch: too many chains or state elements");
  return guarded([&] {
    DeviceGuard g(ctx->device);
    std::unique_ptr<gbm_target> t(new gbm_target());
    t->ctx = ctx;
    t->impl = gbm::make_batch(ctx, m, count);
    finish_target(ctx, t.get(), out);
    t.release();
    return GBM_OK;
  });
}

int gbm_target_transformed(gbm_target* inner, const int32_t* bijector, gbm_target** out) {
  if (!inner || !bijector || !out) return invalid("gbm_target_transformed: NULL argument");
  if (inner->impl->ragged_chains())
    return invalid("gbm_target_transformed: batch targets are not supported");
  for (int64_t d = 0; d < inner->impl->dim; ++d)
    if (bijector[d] < GBM_BIJECTOR_IDENTITY || bijector[d] > GBM_BIJECTOR_SIGMOID)
      return invalid("gbm_target_transformed: bijector codes are GBM_BIJECTOR_*");
  gbm_context* ctx = inner->ctx;
  return guarded([&] {
    DeviceGuard g(ctx->device);
    std::unique_ptr<gbm_target> t(new gbm_target());
    t->ctx = ctx;
    t->impl = gbm::make_transformed(ctx, inner->impl.get(), bijector);
    finish_target(ctx, t.get(), out);
    t.release();
    return GBM_OK;
  });
}

int gbm_target_batch_layout(const gbm_target* t, int64_t* offsets, int32_t* dims,
                            int64_t* chains, int64_t* elements) {
  if (!t) return invalid("gbm_target_batch_layout: NULL target");
  const int64_t C = t->impl->ragged_chains();
  if (C == 0) return invalid("gbm_target_batch_layout: not a batch target");
  return guarded([&] {
    DeviceGuard g(t->ctx->device);
    if (offsets)
      GBM_CUDA(cudaMemcpy(offsets, t->impl->ragged_offsets(), sizeof(int64_t) * C,
                          cudaMemcpyDeviceToHost));
    if (dims)
      GBM_CUDA(cudaMemcpy(dims, t->impl->ragged_dims(), sizeof(int32_t) * C,
                          cudaMemcpyDeviceToHost));
    if (chains) *chains = C;
    if (elements) *elements = t->impl->ragged_elements();
    return GBM_OK;
  });
}

int gbm_target_batch_schedule(const gbm_target* t, int32_t chain_tile[4]) {
  if (!t || !chain_tile) return invalid("gbm_target_batch_schedule: NULL argument");
  if (!gbm::batch_schedule(t->impl.get(), chain_tile))
    return invalid("gbm_target_batch_schedule: not a batch target");
  return GBM_OK;
}

int gbm_target_destroy(gbm_target* t) {
  if (!t) return GBM_OK;
  return guarded([&] {
    DeviceGuard g(t->ctx->device);
    cudaStreamSynchronize(t->ctx->stream);
    delete t;
    return GBM_OK;
  });
}

int gbm_target_dim(const gbm_target* t, int64_t* dim) {
  if (!t || !dim) return invalid("gbm_target_dim: NULL argument");
  *dim = t->impl->dim;
  return GBM_OK;
}

int gbm_target_cost(const gbm_target* t, int64_t chains, double* flops, double* bytes) {
  if (!t || !flops || !bytes) return invalid("gbm_target_cost: NULL argument");
  *flops = t->impl->flops(chains);
  *bytes = t->impl->bytes(chains);
  return GBM_OK;
}

int gbm_target_log_prob_and_grad(gbm_target* t, const float* state, int64_t chains,
                                 double* log_prob, float* grad) {
  if (!t || !state || !log_prob || !grad) return invalid("gbm_target_log_prob_and_grad: NULL argument");
  if (chains <= 0 || chains > (1 << 24)) return invalid("gbm_target_log_prob_and_grad: bad chains");
  return guarded([&] {
    DeviceGuard g(t->ctx->device);
    cudaStream_t s = t->ctx->stream;
    gbm::check_device_error(t->ctx);
    const size_t need = t->impl->workspace_bytes(chains);
    if (need > t->ws.bytes) {
      // The workspace is about to be replaced: let earlier calls finish.
      GBM_CUDA(cudaStreamSynchronize(s));
      t->ws.reserve(need);
    }
    const int n = (int)chains;
    if (t->impl->ragged_chains() && chains != t->impl->ragged_chains())
      return invalid("gbm_target_log_prob_and_grad: a batch target evaluates all its chains");
    gbm::set_count(t->count.as<int>(), n, s);
    t->impl->eval(state, (int)t->impl->dim, t->count.as<int>(), n, log_prob, grad,
                  (int)t->impl->dim, t->ws.ptr, s);
    return GBM_OK;
  });
}

int gbm_hmc_create(gbm_target* target, int64_t max_chains, gbm_hmc** out) {
  if (!target || !out) return invalid("gbm_hmc_create: NULL argument");
  if (max_chains <= 0 || max_chains > (1 << 24)) return invalid("gbm_hmc_create: bad max_chains");
  return guarded([&] {
    DeviceGuard g(target->ctx->device);
    auto* k = new gbm_hmc();
    k->target = target;
    k->ctx = target->ctx;
    k->max_chains = max_chains;
    try {
      gbm::hmc_setup(k);
    } catch (...) {
      delete k;
      throw;
    }
    *out = k;
    return GBM_OK;
  });
}

int gbm_hmc_destroy(gbm_hmc* k) {
  if (!k) return GBM_OK;
  return guarded([&] {
    // Uses only the handle's own context: the target may already be gone.
    DeviceGuard g(k->ctx->device);
    cudaStreamSynchronize(k->ctx->stream);
    delete k;
    return GBM_OK;
  });
}

int gbm_hmc_one_step(gbm_hmc* k, int64_t chains, const float* state,
                     const double* target_log_prob, const float* grads,
                     const float* step_size, int step_size_per_chain,
                     int32_t num_leapfrog_steps, const uint32_t seed[2],
                     float* next_state, double* next_tlp, float* next_grads,
                     float* proposed_state, double* proposed_tlp, float* proposed_grads,
                     float* initial_momentum, float* final_momentum,
                     double* log_acceptance_correction, double* log_accept_ratio,
                     uint8_t* is_accepted) {
  if (!k || !state || !target_log_prob || !grads || !step_size || !seed || !next_state ||
      !next_tlp || !next_grads || !log_accept_ratio || !is_accepted)
    return invalid("gbm_hmc_one_step: NULL argument");
  if (chains <= 0 || chains > k->max_chains)
    return invalid("gbm_hmc_one_step: chains must be in [1, max_chains]");
  if (num_leapfrog_steps < 1) return invalid("gbm_hmc_one_step: num_leapfrog_steps must be >= 1");
  return guarded([&] {
    DeviceGuard g(k->target->ctx->device);
    gbm::check_device_error(k->target->ctx);
    gbm::HmcOutputs out{next_state, next_tlp, next_grads, proposed_state, proposed_tlp,
                        proposed_grads, initial_momentum, final_momentum,
                        log_acceptance_correction, log_accept_ratio, is_accepted};
    gbm::hmc_one_step(k, chains, state, target_log_prob, grads, step_size, step_size_per_chain,
                      num_leapfrog_steps, make_uint2(seed[0], seed[1]), out);
    return GBM_OK;
  });
}

int gbm_nuts_create(gbm_target* target, int64_t max_chains, int32_t max_tree_depth,
                    double max_energy_diff, int32_t unrolled_leapfrog_steps, gbm_nuts** out) {
  if (!target || !out) return invalid("gbm_nuts_create: NULL argument");
  if (max_tree_depth < 1 || max_tree_depth > 16)
    return invalid("max_tree_depth must be known statically and >= 1 (engine limit 16)");
  if (max_chains <= 0 || max_chains > (1 << 24)) return invalid("gbm_nuts_create: bad max_chains");
  if (unrolled_leapfrog_steps < 1) return invalid("gbm_nuts_create: unrolled_leapfrog_steps < 1");
  if (target->impl->ragged_chains() && max_chains != target->impl->ragged_chains())
    return invalid("gbm_nuts_create: a batch target's sampler runs exactly its chains");
  return guarded([&] {
    DeviceGuard g(target->ctx->device);
    auto* k = new gbm_nuts();
    k->target = target;
    k->ctx = target->ctx;
    k->max_chains = max_chains;
    k->max_tree_depth = max_tree_depth;
    k->max_energy_diff = max_energy_diff;
    k->unrolled_leapfrog_steps = unrolled_leapfrog_steps;
    try {
      gbm::nuts_setup(k);
    } catch (...) {
      delete k;
      throw;
    }
    *out = k;
    return GBM_OK;
  });
}

int gbm_nuts_destroy(gbm_nuts* k) {
  if (!k) return GBM_OK;
  return guarded([&] {
    // Uses only the handle's own context: the target may already be gone.
    DeviceGuard g(k->ctx->device);
    cudaStreamSynchronize(k->ctx->stream);
    for (auto& ev : k->poll_events)
      if (ev) cudaEventDestroy(ev);
    for (auto& ev : k->prof_events) cudaEventDestroy(ev);
    gbm::nuts_release_graphs(k);
    delete k;
    return GBM_OK;
  });
}

int gbm_nuts_one_step(gbm_nuts* k, int64_t chains, const float* state,
                      const double* target_log_prob, const float* grads,
                      const float* step_size, int step_size_per_chain, const uint32_t seed[2],
                      float* next_state, double* next_tlp, float* next_grads,
                      double* log_accept_ratio, int32_t* leapfrogs_taken, uint8_t* is_accepted,
                      uint8_t* reach_max_depth, uint8_t* has_divergence, double* energy,
                      int32_t* tree_depth) {
  if (!k || !state || !target_log_prob || !grads || !step_size || !seed || !next_state ||
      !next_tlp || !next_grads || !log_accept_ratio || !leapfrogs_taken || !is_accepted ||
      !reach_max_depth || !has_divergence || !energy)
    return invalid("gbm_nuts_one_step: NULL argument");
  if (chains <= 0 || chains > k->max_chains)
    return invalid("gbm_nuts_one_step: chains must be in [1, max_chains]");
  if (k->dev.ragged && chains != k->max_chains)
    return invalid("gbm_nuts_one_step: a batch target's sampler steps all its chains");
  return guarded([&] {
    DeviceGuard g(k->target->ctx->device);
    gbm::NutsOutputs out{next_state, next_tlp, next_grads, log_accept_ratio, leapfrogs_taken,
                         is_accepted, reach_max_depth, has_divergence, energy, tree_depth};
    gbm::nuts_one_step(k, chains, state, target_log_prob, grads, step_size, step_size_per_chain,
                       make_uint2(seed[0], seed[1]), out);
    return GBM_OK;
  });
}

int gbm_nuts_run_free(gbm_nuts* k, int64_t chains, const float* state,
                      const double* target_log_prob, const float* grads,
                      const float* step_size, int step_size_per_chain, const uint32_t seed[2],
                      int64_t first_step, int32_t transitions_per_chain,
                      int64_t max_leaf_iterations, int32_t* transitions_done,
                      float* trace_state, double* trace_target_log_prob,
                      double* trace_log_accept_ratio, int32_t* trace_leapfrogs_taken,
                      uint8_t* trace_is_accepted, uint8_t* trace_has_divergence,
                      int64_t* leaf_iterations) {
  if (!k || !state || !target_log_prob || !grads || !step_size || !seed)
    return invalid("gbm_nuts_run_free: NULL argument");
  if (chains <= 0 || chains > k->max_chains)
    return invalid("gbm_nuts_run_free: chains must be in [1, max_chains]");
  if (k->dev.ragged && chains != k->target->impl->ragged_chains())
    return invalid("gbm_nuts_run_free: a batch target's sampler runs exactly its chains");
  if (transitions_per_chain < 1 || max_leaf_iterations < 1)
    return invalid("gbm_nuts_run_free: need transitions_per_chain >= 1 and "
                   "max_leaf_iterations >= 1");
  if (k->unrolled_leapfrog_steps != 1)
    return invalid("gbm_nuts_run_free: needs unrolled_leapfrog_steps == 1");
  if (first_step < 0 || first_step + transitions_per_chain > ((int64_t)1 << 32))
    return invalid("gbm_nuts_run_free: step indices must fit 32 bits");
  return guarded([&] {
    DeviceGuard g(k->target->ctx->device);
    gbm::check_device_error(k->target->ctx);
    gbm::FreeDev f{};
    f.tr_state = trace_state;
    f.tr_logp = trace_target_log_prob;
    f.tr_lar = trace_log_accept_ratio;
    f.tr_lf = trace_leapfrogs_taken;
    f.tr_acc = trace_is_accepted;
    f.tr_div = trace_has_divergence;
    f.tr_estride = k->dev.ragged ? (size_t)k->target->impl->ragged_elements()
                                 : (size_t)chains * (size_t)k->target->impl->dim;
    const int64_t it = gbm::nuts_run_free(
        k, chains, state, target_log_prob, grads, step_size, step_size_per_chain,
        make_uint2(seed[0], seed[1]), (uint32_t)first_step, transitions_per_chain,
        max_leaf_iterations, f, transitions_done);
    if (leaf_iterations) *leaf_iterations = it;
    return GBM_OK;
  });
}

int gbm_nuts_last_leaf_iterations(const gbm_nuts* k, int64_t* out) {
  if (!k || !out) return invalid("gbm_nuts_last_leaf_iterations: NULL argument");
  *out = k->last_leaf_iterations;
  return GBM_OK;
}

static int check_loop_args(int64_t chains, int64_t max_chains, int64_t first_step,
                           int64_t num_results, int64_t burnin, int64_t thin,
                           int32_t num_adaptation_steps, const double* da_state) {
  if (chains <= 0 || chains > max_chains) return invalid("sample_chain: chains must be in [1, max_chains]");
  if (num_results < 1 || burnin < 0 || thin < 0 || first_step < 0)
    return invalid("sample_chain: need num_results >= 1, burn-in, thinning, first_step >= 0");
  const int64_t total = first_step + burnin + 1 + (num_results - 1) * (1 + thin);
  if (total >= ((int64_t)1 << 32)) return invalid("sample_chain: more than 2^32 transitions");
  if (num_adaptation_steps > 0 && !da_state)
    return invalid("sample_chain: adaptation needs da_state");
  return GBM_OK;
}

int gbm_nuts_sample_chain(gbm_nuts* k, int64_t chains, float* state, double* tlp, float* grads,
                          float* step_size, int per_chain, const uint32_t seed[2],
                          int64_t first_step, int64_t num_results, int64_t burnin, int64_t thin,
                          int32_t num_adaptation_steps, double target_accept_prob,
                          double exploration_shrinkage, double step_count_smoothing,
                          double decay_rate, double* da_state, float* trace_state,
                          double* trace_tlp, double* trace_lar, int32_t* trace_lf,
                          uint8_t* trace_acc, uint8_t* trace_div, float* trace_eps) {
  if (!k || !state || !tlp || !grads || !step_size || !seed)
    return invalid("gbm_nuts_sample_chain: NULL argument");
  const int st = check_loop_args(chains, k->max_chains, first_step, num_results, burnin, thin,
                                 num_adaptation_steps, da_state);
  if (st != GBM_OK) return st;
  return guarded([&] {
    DeviceGuard g(k->target->ctx->device);
    gbm::check_device_error(k->target->ctx);
    gbm::DaConfig da{num_adaptation_steps > 0 ? 1 : 0,
                     gbm::DaParams{target_accept_prob, exploration_shrinkage,
                                   step_count_smoothing, decay_rate, num_adaptation_steps},
                     nullptr, da_state};
    gbm::ChainTrace tr{trace_state, trace_tlp, trace_lar, trace_lf, trace_acc, trace_div,
                       trace_eps, nullptr, nullptr};
    gbm::nuts_sample_chain(k, chains, state, tlp, grads, step_size, per_chain,
                           make_uint2(seed[0], seed[1]), (uint32_t)first_step, num_results,
                           burnin, thin, da, tr);
    return GBM_OK;
  });
}

int gbm_hmc_sample_chain(gbm_hmc* k, int64_t chains, float* state, double* tlp, float* grads,
                         float* step_size, int per_chain, int32_t num_leapfrog_steps,
                         const uint32_t seed[2], int64_t first_step, int64_t num_results,
                         int64_t burnin, int64_t thin, int32_t num_adaptation_steps,
                         double target_accept_prob, double exploration_shrinkage,
                         double step_count_smoothing, double decay_rate, double* da_state,
                         float* trace_state, double* trace_tlp, double* trace_lar,
                         uint8_t* trace_acc, float* trace_eps) {
  if (!k || !state || !tlp || !grads || !step_size || !seed)
    return invalid("gbm_hmc_sample_chain: NULL argument");
  if (num_leapfrog_steps < 1) return invalid("gbm_hmc_sample_chain: num_leapfrog_steps < 1");
  const int st = check_loop_args(chains, k->max_chains, first_step, num_results, burnin, thin,
                                 num_adaptation_steps, da_state);
  if (st != GBM_OK) return st;
  return guarded([&] {
    DeviceGuard g(k->target->ctx->device);
    gbm::check_device_error(k->target->ctx);
    gbm::DaConfig da{num_adaptation_steps > 0 ? 1 : 0,
                     gbm::DaParams{target_accept_prob, exploration_shrinkage,
                                   step_count_smoothing, decay_rate, num_adaptation_steps},
                     nullptr, da_state};
    gbm::ChainTrace tr{trace_state, trace_tlp, trace_lar, nullptr, trace_acc, nullptr, trace_eps,
                       nullptr, nullptr};
    gbm::hmc_sample_chain(k, chains, state, tlp, grads, step_size, per_chain, num_leapfrog_steps,
                          make_uint2(seed[0], seed[1]), (uint32_t)first_step, num_results, burnin,
                          thin, da, tr);
    return GBM_OK;
  });
}

int gbm_nuts_set_profiling(gbm_nuts* k, int enable) {
  if (!k) return invalid("gbm_nuts_set_profiling: NULL argument");
  k->profiling = enable != 0;
  return GBM_OK;
}

int gbm_moments_update(gbm_context* ctx, const float* state, int64_t elements,
                       int64_t count_before, double* mean, double* m2) {
  if (!ctx || !state || !mean || !m2) return invalid("gbm_moments_update: NULL argument");
  if (elements <= 0 || count_before < 0) return invalid("gbm_moments_update: bad sizes");
  return guarded([&] {
    DeviceGuard g(ctx->device);
    gbm::moments_update(ctx->stream, state, (size_t)elements, count_before, mean, m2);
    return GBM_OK;
  });
}

int gbm_autocov_update(gbm_context* ctx, const float* state, int64_t elements,
                       int64_t count_before, int32_t max_lag, float* first, double* total,
                       float* head, float* ring, double* lag_sums) {
  if (!ctx || !state || !first || !total || !head || !ring || !lag_sums)
    return invalid("gbm_autocov_update: NULL argument");
  if (elements <= 0 || count_before < 0 || max_lag < 1 || max_lag > 4096)
    return invalid("gbm_autocov_update: bad sizes (1 <= max_lag <= 4096)");
  return guarded([&] {
    DeviceGuard g(ctx->device);
    gbm::autocov_update(ctx->stream, state, (size_t)elements, count_before, max_lag, first,
                        total, head, ring, lag_sums);
    return GBM_OK;
  });
}

int gbm_nuts_set_graphs(gbm_nuts* k, int enable) {
  if (!k) return invalid("gbm_nuts_set_graphs: NULL argument");
  k->use_graphs = enable != 0;
  return GBM_OK;
}

int gbm_nuts_set_free_running(gbm_nuts* k, int enable) {
  if (!k) return invalid("gbm_nuts_set_free_running: NULL argument");
  k->free_draws = enable != 0;
  return GBM_OK;
}

int gbm_nuts_set_inverse_mass(gbm_nuts* k, const float* inverse_mass, int per_chain) {
  if (!k) return invalid("gbm_nuts_set_inverse_mass: NULL kernel");
  if (k->dev.ragged && inverse_mass && !per_chain)
    return invalid("gbm_nuts_set_inverse_mass: batch targets need a per-chain (ragged) array");
  return guarded([&] {
    if (k->inv_mass != inverse_mass || k->im_per_chain != (per_chain != 0)) {
      // Captured graphs hold the pointer: capture again.
      GBM_CUDA(cudaStreamSynchronize(k->ctx->stream));
      gbm::nuts_clear_graphs(k);
    }
    k->inv_mass = inverse_mass;
    k->im_per_chain = per_chain != 0;
    return GBM_OK;
  });
}

int gbm_nuts_read_profile(gbm_nuts* k, double* eval_ms, int64_t* evals, int64_t* launches) {
  if (!k || !eval_ms || !evals || !launches) return invalid("gbm_nuts_read_profile: NULL argument");
  return guarded([&] {
    DeviceGuard g(k->target->ctx->device);
    GBM_CUDA(cudaStreamSynchronize(k->target->ctx->stream));
    gbm::nuts_profile_flush(k);
    *eval_ms = k->prof_eval_ms;
    *evals = k->prof_evals;
    *launches = k->prof_launches;
    k->prof_eval_ms = 0.0;
    k->prof_evals = 0;
    k->prof_launches = 0;
    return GBM_OK;
  });
}

int gbm_dual_averaging_update(gbm_context* ctx, int64_t chains, const double* lar, int per_chain,
                              int32_t num_adaptation_steps, double target_accept_scalar,
                              const double* target_accept_prob, double exploration_shrinkage,
                              double step_count_smoothing, double decay_rate, double* state,
                              float* step_size) {
  if (!ctx || !lar || !state || !step_size) return invalid("gbm_dual_averaging_update: NULL argument");
  if (chains <= 0) return invalid("gbm_dual_averaging_update: chains must be > 0");
  return guarded([&] {
    DeviceGuard g(ctx->device);
    gbm::DaParams prm{target_accept_scalar, exploration_shrinkage, step_count_smoothing,
                      decay_rate, num_adaptation_steps};
    gbm::dual_averaging_update(ctx->stream, lar, chains, per_chain, prm, target_accept_prob,
                               state, step_size);
    return GBM_OK;
  });
}

int gbm_dual_averaging_update_reduced(gbm_context* ctx, int64_t groups,
                                      const double* reduced_log_accept_prob,
                                      int32_t num_adaptation_steps, double target_accept_scalar,
                                      const double* target_accept_prob,
                                      double exploration_shrinkage, double step_count_smoothing,
                                      double decay_rate, double* state, float* step_size) {
  if (!ctx || !reduced_log_accept_prob || !state || !step_size)
    return invalid("gbm_dual_averaging_update_reduced: NULL argument");
  if (groups <= 0) return invalid("gbm_dual_averaging_update_reduced: groups must be > 0");
  return guarded([&] {
    DeviceGuard g(ctx->device);
    gbm::DaParams prm{target_accept_scalar, exploration_shrinkage, step_count_smoothing,
                      decay_rate, num_adaptation_steps};
    gbm::dual_averaging_update_reduced(ctx->stream, reduced_log_accept_prob, groups, prm,
                                       target_accept_prob, state, step_size);
    return GBM_OK;
  });
}

int gbm_metropolis_hastings_step(gbm_context* ctx, int64_t chains, int64_t dim,
                                 const uint32_t seed[2], const double* current_target_log_prob,
                                 const double* proposed_target_log_prob,
                                 const double* log_acceptance_correction,
                                 const float* current_state, const float* proposed_state,
                                 float* next_state, double* log_accept_ratio,
                                 uint8_t* is_accepted) {
  if (!ctx || !seed || !current_target_log_prob || !proposed_target_log_prob ||
      !current_state || !proposed_state || !next_state || !log_accept_ratio || !is_accepted)
    return invalid("gbm_metropolis_hastings_step: NULL argument");
  if (chains <= 0 || chains > (1 << 24) || dim <= 0)
    return invalid("gbm_metropolis_hastings_step: bad chains or dim");
  return guarded([&] {
    DeviceGuard g(ctx->device);
    gbm::metropolis_hastings_step(ctx->stream, chains, dim, make_uint2(seed[0], seed[1]),
                                  current_target_log_prob, proposed_target_log_prob,
                                  log_acceptance_correction, current_state, proposed_state,
                                  next_state, log_accept_ratio, is_accepted);
    return GBM_OK;
  });
}

}  // extern "C"
