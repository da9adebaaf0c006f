// Job server: many independent DA(NUTS) posteriors running concurrently.
//
// Each worker thread owns two contexts on private non-blocking streams (one
// of the device's greatest priority, one of its least) and runs one job at a
// time to completion on one of them: build the target on its stream,
// evaluate the initial state, run the device-resident chain loop
// (nuts_sample_chain: dual averaging, then the draws past its window
// free-running) with the requested trace, copy the final state out, free
// everything.  Jobs with little work per leaf take the high-priority stream.
// Buffers come from the stream-ordered allocator (alloc_stream()), so a
// job's set-up and tear-down do not synchronize the device and the other
// workers' kernels keep running.  Admission is first-in first-out under a
// device-memory budget.
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <thread>
#include <unordered_map>
#include <vector>

#include "gb300_mcmc.h"
#include "samplers.h"

namespace gbm {

std::unique_ptr<Target> make_logreg_tc(gbm_context* ctx, const void* X, int x_dtype, int64_t n,
                                       int64_t d, const float* y, float prior_scale);

namespace {

__global__ void init_loop_state(float* eps, double* da_state, float step) {
  eps[0] = step;
  da_state[0] = 0.0;
  da_state[1] = 0.0;
  da_state[2] = log(10.0) + log((double)step);   // log(10 * initial step), :588-590
  da_state[3] = 0.0;
}

struct Job {
  gbm_job_spec spec;
  int64_t id = 0;
  int status = GBM_JOB_QUEUED;
  int error_code = GBM_OK;
  std::string error;
  size_t bytes = 0;
  double t_submit = 0, t_start = 0, t_end = 0;
};

int family_dim(const gbm_job_spec& s, int64_t* dim) {
  switch (s.family) {
    case GBM_FAMILY_LOGISTIC_REGRESSION: *dim = s.features; return GBM_OK;
    case GBM_FAMILY_MVN: *dim = s.dim; return GBM_OK;
    case GBM_FAMILY_HIERARCHICAL_NORMAL: *dim = s.groups + 2; return GBM_OK;
    default: return GBM_EINVAL;
  }
}

// Device memory a job needs (target data + workspaces + NUTS + loop buffers).
size_t estimate_bytes(const gbm_job_spec& s, int num_sms) {
  const double C = (double)s.chains, D = (double)s.dim;
  double b = 0;
  if (s.family == GBM_FAMILY_LOGISTIC_REGRESSION) {
    const double N = (double)s.rows;
    const double Dp = std::ceil(D / 64.0) * 64.0;
    const bool mixed = s.precision == GBM_PRECISION_MIXED;
    b += mixed ? N * Dp * 4.0 : N * (std::ceil(D / 16.0) * 16.0) * 4.0;
    b += N * 8.0;
    b += (2.0 * num_sms * 128.0 + C) * (8.0 + 4.0 * D);
    if (D > (mixed ? 512.0 : 256.0))   // library-GEMM target: Z and R (hi, lo), B, G, cuBLAS
      b += (N + 8.0) * C * (mixed ? 12.0 : 8.0) + C * Dp * 16.0 + (32u << 20);
  } else if (s.family == GBM_FAMILY_MVN) {
    b += 4.0 * D * D + 4.0 * D + C * (8.0 * std::ceil(D / 64.0) + 4.0 * D);
  } else {
    b += 8.0 * (double)s.groups;
  }
  const double vec = C * D;
  b += 4.0 * vec * (14.0 + 2.0 * s.max_tree_depth) + 160.0 * C;   // NUTS workspace
  b += 8.0 * vec + 64.0 * C;                                        // chain loop buffers
  b += 8.0 * vec + 16.0 * C;                                        // job state
  // Free-running draws: leaf tables, per-chain loop state and, when the job
  // traces no log-accept ratios, their rows for the dual-averaging replay.
  b += 12.0 * (double)(1 << s.max_tree_depth) + 32.0 * C;
  if (!s.trace_log_accept_ratio) b += 8.0 * C * (double)s.num_results;
  return (size_t)b + (1u << 20);
}

}  // namespace
}  // namespace gbm

struct gbm_server {
  int device = 0;
  size_t budget = 0;
  size_t in_use = 0;
  int num_sms = 0;
  bool stopping = false;
  int64_t next_id = 1;
  std::chrono::steady_clock::time_point t0;
  std::mutex mu;
  std::condition_variable work_cv, done_cv;
  std::deque<gbm::Job*> queue;
  std::unordered_map<int64_t, std::unique_ptr<gbm::Job>> jobs;
  std::vector<std::thread> workers;

  double now() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
};

namespace gbm {
namespace {

void run_job(gbm_context* ctx, Job* job) {
  const gbm_job_spec& s = job->spec;
  cudaStream_t st = ctx->stream;
  std::unique_ptr<gbm_target> t(new gbm_target());
  t->ctx = ctx;
  switch (s.family) {
    case GBM_FAMILY_LOGISTIC_REGRESSION:
      t->impl = s.precision == GBM_PRECISION_MIXED
                    ? make_logreg_tc(ctx, s.x, s.x_dtype, s.rows, s.features, s.y, s.prior_scale)
                    : make_logreg_simt(ctx, static_cast<const float*>(s.x), s.rows, s.features,
                                       s.y, s.prior_scale);
      if (!t->impl)   // beyond the fused kernels' feature limits
        t->impl = make_logreg_large(ctx, s.x, s.x_dtype, s.rows, s.features, s.y,
                                    s.prior_scale, s.precision == GBM_PRECISION_MIXED);
      break;
    case GBM_FAMILY_MVN:
      t->impl = make_mvn(ctx, s.loc, s.scale_tril_inv, s.dim, s.log_normalizer);
      break;
    default:
      t->impl = make_hier(ctx, s.group_y, s.group_sigma, s.groups, s.mu_scale, s.tau_scale);
  }
  if (!t->impl) throw std::runtime_error("job target unavailable for this shape/precision");
  t->count.reserve(sizeof(int));
  const int64_t C = s.chains, D = s.dim;
  gbm_nuts k;
  k.target = t.get();
  k.ctx = ctx;
  k.max_chains = C;
  k.max_tree_depth = s.max_tree_depth;
  k.max_energy_diff = 1000.0;
  k.unrolled_leapfrog_steps = 1;
  k.free_draws = true;   // draws after adaptation: no chain waits for another's trajectory
  nuts_setup(&k);
  DeviceBuffer q, l, g, eps, da;
  q.reserve(sizeof(float) * C * D);
  g.reserve(sizeof(float) * C * D);
  l.reserve(sizeof(double) * C);
  eps.reserve(256);
  da.reserve(256);
  GBM_CUDA(cudaMemcpyAsync(q.ptr, s.init_state, sizeof(float) * C * D, cudaMemcpyDeviceToDevice,
                           st));
  t->ws.reserve(t->impl->workspace_bytes(C));
  set_count(t->count.as<int>(), (int)C, st);
  t->impl->eval(q.as<float>(), (int)D, t->count.as<int>(), (int)C, l.as<double>(), g.as<float>(),
                (int)D, t->ws.ptr, st);
  init_loop_state<<<1, 1, 0, st>>>(eps.as<float>(), da.as<double>(), s.step_size);
  GBM_CUDA(cudaGetLastError());
  DaConfig dac{s.num_adaptation_steps > 0 ? 1 : 0,
               DaParams{s.target_accept_prob, 0.05, 10.0, 0.75, s.num_adaptation_steps}, nullptr,
               da.as<double>()};
  ChainTrace tr{s.trace_state, nullptr, s.trace_log_accept_ratio, s.trace_leapfrogs_taken,
                nullptr, nullptr, nullptr, s.moments_mean, s.moments_m2};
  if (s.moments_mean && s.moments_m2) {
    GBM_CUDA(cudaMemsetAsync(s.moments_mean, 0, sizeof(double) * C * D, st));
    GBM_CUDA(cudaMemsetAsync(s.moments_m2, 0, sizeof(double) * C * D, st));
  }
  nuts_sample_chain(&k, C, q.as<float>(), l.as<double>(), g.as<float>(), eps.as<float>(), 0,
                    make_uint2(s.seed[0], s.seed[1]), 0, s.num_results, s.num_burnin_steps, 0, dac,
                    tr);
  if (s.final_state)
    GBM_CUDA(cudaMemcpyAsync(s.final_state, q.ptr, sizeof(float) * C * D,
                             cudaMemcpyDeviceToDevice, st));
  if (s.final_step_size)
    GBM_CUDA(cudaMemcpyAsync(s.final_step_size, eps.ptr, sizeof(float), cudaMemcpyDeviceToDevice,
                             st));
  GBM_CUDA(cudaStreamSynchronize(st));
  check_device_error(ctx);
  for (auto& ev : k.poll_events)
    if (ev) cudaEventDestroy(ev);
  for (auto& ev : k.prof_events) cudaEventDestroy(ev);
  nuts_release_graphs(&k);
}

// Multiply-adds of one batched gradient evaluation of the job's chains.
double leaf_work(const gbm_job_spec& s) {
  const double C = (double)s.chains;
  switch (s.family) {
    case GBM_FAMILY_LOGISTIC_REGRESSION: return (double)s.rows * (double)s.features * C;
    case GBM_FAMILY_MVN: return (double)s.dim * (double)s.dim * C;
    default: return 10.0 * (double)s.groups * C;
  }
}

// Jobs below this much work per leaf run on the worker's high-priority
// stream: their kernels' blocks are scheduled ahead of the large jobs'
// pending blocks whenever SMs free up, so a few large jobs do not multiply
// the latency of every small one.
constexpr double kSmallLeafWork = 2e9;

void worker_main(gbm_server* srv) {
  cudaSetDevice(srv->device);
  gbm_context ctx_hi, ctx_lo;
  try {
    int least = 0, greatest = 0;
    GBM_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    cudaStream_t s_hi = nullptr, s_lo = nullptr;
    GBM_CUDA(cudaStreamCreateWithPriority(&s_hi, cudaStreamNonBlocking, greatest));
    context_init(&ctx_hi, srv->device, s_hi, true);
    GBM_CUDA(cudaStreamCreateWithPriority(&s_lo, cudaStreamNonBlocking, least));
    context_init(&ctx_lo, srv->device, s_lo, true);
  } catch (...) {
    context_free(&ctx_hi);
    context_free(&ctx_lo);
    return;
  }
  while (true) {
    Job* job = nullptr;
    {
      std::unique_lock<std::mutex> lock(srv->mu);
      srv->work_cv.wait(lock, [&] {
        return srv->stopping ||
               (!srv->queue.empty() &&
                (srv->in_use == 0 || srv->in_use + srv->queue.front()->bytes <= srv->budget));
      });
      if (srv->stopping) break;
      job = srv->queue.front();
      srv->queue.pop_front();
      srv->in_use += job->bytes;
      job->status = GBM_JOB_RUNNING;
      job->t_start = srv->now();
    }
    int code = GBM_OK;
    std::string msg;
    gbm_context* ctx = leaf_work(job->spec) < kSmallLeafWork ? &ctx_hi : &ctx_lo;
    alloc_stream() = ctx->stream;
    try {
      run_job(ctx, job);
    } catch (const CudaError& e) {
      code = e.err == cudaErrorMemoryAllocation ? GBM_ENOMEM : GBM_ECUDA;
      msg = std::string(e.what) + ": " + cudaGetErrorString(e.err);
    } catch (const DeviceTimeout& e) {
      code = GBM_ETIMEDOUT;
      msg = "bounded device wait timed out (code " + std::to_string(e.code) + ")";
    } catch (const std::exception& e) {
      code = GBM_ENOTSUP;
      msg = e.what();
    }
    if (code != GBM_OK) cudaStreamSynchronize(ctx->stream);
    {
      std::lock_guard<std::mutex> lock(srv->mu);
      srv->in_use -= job->bytes;
      job->t_end = srv->now();
      job->status = code == GBM_OK ? GBM_JOB_DONE : GBM_JOB_FAILED;
      job->error_code = code;
      job->error = msg;
    }
    srv->done_cv.notify_all();
    srv->work_cv.notify_all();
  }
  alloc_stream() = nullptr;
  context_free(&ctx_hi);
  context_free(&ctx_lo);
}

void fill_info(const Job* j, gbm_job_info* info) {
  if (!info) return;
  info->status = j->status;
  info->error_code = j->error_code;
  info->submit_s = j->t_submit;
  info->start_s = j->t_start;
  info->end_s = j->t_end;
  info->device_bytes = (int64_t)j->bytes;
}

}  // namespace
}  // namespace gbm

extern "C" {

int gbm_server_create(int device, int32_t workers, int64_t budget, gbm_server** out) {
  if (!out || workers < 1 || workers > 256 || budget <= 0) {
    gbm::set_error("gbm_server_create: need out, 1 <= workers <= 256, budget > 0");
    return GBM_EINVAL;
  }
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) {
    gbm::set_error("gbm_server_create: bad device index");
    return GBM_EINVAL;
  }
  auto* srv = new gbm_server();
  srv->device = device;
  srv->budget = (size_t)budget;
  srv->t0 = std::chrono::steady_clock::now();
  cudaDeviceGetAttribute(&srv->num_sms, cudaDevAttrMultiProcessorCount, device);
  // Keep freed job memory in the stream-ordered pool instead of returning it.
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t keep = (uint64_t)budget;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  for (int i = 0; i < workers; ++i) srv->workers.emplace_back(gbm::worker_main, srv);
  *out = srv;
  return GBM_OK;
}

int gbm_server_destroy(gbm_server* srv) {
  if (!srv) return GBM_OK;
  {
    std::lock_guard<std::mutex> lock(srv->mu);
    srv->stopping = true;
    srv->queue.clear();
  }
  srv->work_cv.notify_all();
  for (auto& t : srv->workers) t.join();
  delete srv;
  return GBM_OK;
}

int gbm_server_submit(gbm_server* srv, const gbm_job_spec* spec, int64_t* job_id) {
  if (!srv || !spec || !job_id) {
    gbm::set_error("gbm_server_submit: NULL argument");
    return GBM_EINVAL;
  }
  const gbm_job_spec& s = *spec;
  int64_t dim = 0;
  if (gbm::family_dim(s, &dim) != GBM_OK || dim != s.dim || s.dim <= 0) {
    gbm::set_error("gbm_server_submit: unknown family or dim does not match the family");
    return GBM_EINVAL;
  }
  if (!s.init_state || s.chains <= 0 || s.num_results < 1 || s.num_burnin_steps < 0 ||
      s.max_tree_depth < 1 || s.max_tree_depth > 16 || !(s.step_size > 0.f)) {
    gbm::set_error("gbm_server_submit: bad sampler settings");
    return GBM_EINVAL;
  }
  if (s.family == GBM_FAMILY_LOGISTIC_REGRESSION &&
      (!s.x || !s.y || s.rows <= 0 || s.features < 1 || !(s.prior_scale > 0.f) ||
       (s.precision == GBM_PRECISION_F32 && s.x_dtype != GBM_DTYPE_F32))) {
    gbm::set_error("gbm_server_submit: logistic regression needs x, y, rows > 0, features > 0, "
                   "a positive prior scale and float32 X for FP32 precision");
    return GBM_EINVAL;
  }
  if (s.family == GBM_FAMILY_MVN && (!s.loc || !s.scale_tril_inv)) {
    gbm::set_error("gbm_server_submit: MVN needs loc and scale_tril_inv");
    return GBM_EINVAL;
  }
  if (s.family == GBM_FAMILY_HIERARCHICAL_NORMAL &&
      (!s.group_y || !s.group_sigma || !(s.mu_scale > 0.f) || !(s.tau_scale > 0.f))) {
    gbm::set_error("gbm_server_submit: hierarchical model needs y, sigma and positive scales");
    return GBM_EINVAL;
  }
  std::unique_ptr<gbm::Job> job(new gbm::Job());
  job->spec = s;
  job->bytes = gbm::estimate_bytes(s, srv->num_sms);
  if (job->bytes > srv->budget) {
    gbm::set_error("gbm_server_submit: job needs more device memory than the server budget");
    return GBM_ENOMEM;
  }
  {
    std::lock_guard<std::mutex> lock(srv->mu);
    if (srv->stopping) {
      gbm::set_error("gbm_server_submit: server is stopping");
      return GBM_EINVAL;
    }
    job->id = srv->next_id++;
    job->t_submit = srv->now();
    *job_id = job->id;
    srv->queue.push_back(job.get());
    srv->jobs[job->id] = std::move(job);
  }
  srv->work_cv.notify_one();
  return GBM_OK;
}

int gbm_server_query(gbm_server* srv, int64_t id, gbm_job_info* info) {
  if (!srv) return GBM_EINVAL;
  std::lock_guard<std::mutex> lock(srv->mu);
  auto it = srv->jobs.find(id);
  if (it == srv->jobs.end()) {
    gbm::set_error("gbm_server_query: unknown job id");
    return GBM_EINVAL;
  }
  gbm::fill_info(it->second.get(), info);
  if (it->second->status == GBM_JOB_FAILED) gbm::set_error(it->second->error);
  return GBM_OK;
}

int gbm_server_wait(gbm_server* srv, int64_t id, double timeout_s, gbm_job_info* info) {
  if (!srv) return GBM_EINVAL;
  std::unique_lock<std::mutex> lock(srv->mu);
  auto it = srv->jobs.find(id);
  if (it == srv->jobs.end()) {
    gbm::set_error("gbm_server_wait: unknown job id");
    return GBM_EINVAL;
  }
  gbm::Job* j = it->second.get();
  const bool ok = srv->done_cv.wait_for(
      lock, std::chrono::duration<double>(timeout_s),
      [&] { return j->status == GBM_JOB_DONE || j->status == GBM_JOB_FAILED; });
  gbm::fill_info(j, info);
  if (!ok) {
    gbm::set_error("gbm_server_wait: timed out");
    return GBM_ETIMEDOUT;
  }
  if (j->status == GBM_JOB_FAILED) gbm::set_error(j->error);
  return GBM_OK;
}

int gbm_server_release(gbm_server* srv, int64_t id) {
  if (!srv) return GBM_EINVAL;
  std::lock_guard<std::mutex> lock(srv->mu);
  auto it = srv->jobs.find(id);
  if (it == srv->jobs.end()) return GBM_OK;
  if (it->second->status == GBM_JOB_QUEUED || it->second->status == GBM_JOB_RUNNING) {
    gbm::set_error("gbm_server_release: job has not finished");
    return GBM_EINVAL;
  }
  srv->jobs.erase(it);
  return GBM_OK;
}

double gbm_server_now(gbm_server* srv) { return srv ? srv->now() : 0.0; }

}  // extern "C"
