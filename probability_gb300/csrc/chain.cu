// Device-resident sample_chain loops (mcmc/sample.py:311-383): burn-in,
// thinning, optional dual-averaging step-size adaptation
// (mcmc/dual_averaging_step_size_adaptation.py:477-532) and the trace, all
// enqueued on the context stream from C++ -- no host language in the loop.
// Transition t uses the key step_key(seed, first_step + t), so a run split
// into several calls (first_step advancing) draws exactly as one long run.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <utility>

#include "rng.cuh"
#include "samplers.h"

namespace gbm {

namespace {

template <class T>
void copy_row(T* dst, const T* src, size_t n, cudaStream_t s) {
  if (dst) GBM_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(T), cudaMemcpyDeviceToDevice, s));
}

// Ping-pong state buffers plus per-transition result buffers for C chains.
struct LoopBuffers {
  float *q, *g;
  double *l, *lar, *energy, *corr;
  int32_t* lf;
  uint8_t *acc, *rmd, *div;
};

LoopBuffers carve(DeviceBuffer& mem, int64_t C, int64_t D) {
  const size_t vec = (size_t)C * D;
  size_t bytes = 0;
  auto take = [&](size_t b) { size_t at = bytes; bytes += (b + 255) / 256 * 256; return at; };
  const size_t oq = take(4 * vec), og = take(4 * vec), ol = take(8 * C), olar = take(8 * C);
  const size_t oe = take(8 * C), oc = take(8 * C), olf = take(4 * C), oa = take(C), orm = take(C),
               od = take(C);
  mem.reserve(bytes);
  char* b = mem.as<char>();
  LoopBuffers r;
  r.q = reinterpret_cast<float*>(b + oq);
  r.g = reinterpret_cast<float*>(b + og);
  r.l = reinterpret_cast<double*>(b + ol);
  r.lar = reinterpret_cast<double*>(b + olar);
  r.energy = reinterpret_cast<double*>(b + oe);
  r.corr = reinterpret_cast<double*>(b + oc);
  r.lf = reinterpret_cast<int32_t*>(b + olf);
  r.acc = reinterpret_cast<uint8_t*>(b + oa);
  r.rmd = reinterpret_cast<uint8_t*>(b + orm);
  r.div = reinterpret_cast<uint8_t*>(b + od);
  return r;
}

}  // namespace

__global__ void moments_update_kernel(const float* __restrict__ x, size_t n, double inv_count,
                                      double* __restrict__ mean, double* __restrict__ m2) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double v = (double)x[i];
  const double delta = v - mean[i];
  const double mnew = mean[i] + delta * inv_count;
  mean[i] = mnew;
  m2[i] += delta * (v - mnew);
}

// Running lagged products for a streaming autocovariance (the effective
// sample size of mcmc/diagnostic.py:203-337 truncated at lag L =
// filter_beyond_lag, without storing draws).  Per element e, draws are shifted
// by the first draw, y_t = x_t - x_0 in float64 (exact for float32 draws;
// autocovariance is shift-invariant and the shift keeps the float64 sums from
// cancelling).  Kept: x_0, total = sum y_t, head[j] = x_j for j < L,
// ring[t mod L] = x_t for the last L draws (float32 draws as given), and
// lag[k] = sum_{t >= k} y_t y_{t-k} for k = 0..L.  Arrays are
// [slot][elements] so each update is coalesced.
__global__ void autocov_update_kernel(const float* __restrict__ x, size_t E, int64_t n, int L,
                                      float* __restrict__ x0, double* __restrict__ total,
                                      float* __restrict__ head, float* __restrict__ ring,
                                      double* __restrict__ lag) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  const float xe = x[e];
  if (n == 0) x0[e] = xe;
  const double base = (double)(n == 0 ? xe : x0[e]);
  const double yd = (double)xe - base;
  total[e] += yd;
  lag[e] += yd * yd;
  const int kmax = n < (int64_t)L ? (int)n : L;
  for (int k = 1; k <= kmax; ++k) {
    const double yk = (double)ring[(size_t)((n - k) % L) * E + e] - base;
    lag[(size_t)k * E + e] += yd * yk;
  }
  if (n < (int64_t)L) head[(size_t)n * E + e] = xe;
  ring[(size_t)(n % L) * E + e] = xe;
}

void autocov_update(cudaStream_t s, const float* x, size_t E, int64_t count_before, int L,
                    float* x0, double* total, float* head, float* ring, double* lag) {
  autocov_update_kernel<<<(unsigned)((E + 255) / 256), 256, 0, s>>>(
      x, E, count_before, L, x0, total, head, ring, lag);
  GBM_CUDA(cudaGetLastError());
}

// The key of the transition at the device-side step counter, then advance it
// (so a captured transition can be replayed for every step).
__global__ void advance_step_key_kernel(uint2 seed, uint32_t* step, uint2* key) {
  *key = step_key(seed, *step);
  *step += 1;
}

__global__ void set_step_kernel(uint32_t* step, uint32_t v) { *step = v; }

void moments_update(cudaStream_t s, const float* x, size_t n, int64_t count_before, double* mean,
                    double* m2) {
  if (!mean || !m2 || n == 0) return;
  moments_update_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(
      x, n, 1.0 / (double)(count_before + 1), mean, m2);
  GBM_CUDA(cudaGetLastError());
}

void nuts_sample_chain(gbm_nuts* k, int64_t C, float* q, double* l, float* g, float* eps,
                       int per_chain, uint2 seed, uint32_t first_step, int64_t num_results,
                       int64_t burnin, int64_t thin, const DaConfig& da, const ChainTrace& tr) {
  cudaStream_t s = k->target->ctx->stream;
  const int64_t D = k->target->impl->dim;
  const size_t vec = (size_t)C * D;
  LoopBuffers b = carve(k->loop_mem, C, D);
  float *cq = q, *cg = g, *nq = b.q, *ng = b.g;
  double *cl = l, *nl = b.l;
  const int64_t groups = per_chain ? C : 1;
  // With free_draws, the results whose transitions all run at the final step
  // size (dual averaging past its window, or none) come from the
  // free-running loop: row r_free onward (no thinning).
  int64_t r_free = num_results;
  if (k->free_draws && thin == 0 && !k->dev.ragged && k->unrolled_leapfrog_steps == 1 &&
      num_results > 0) {
    int64_t adapt_end = 0;   // first transition of this call past the window
    if (da.enabled) {
      double step0 = 0.0;   // the window counter (state[3]) at the call's start
      GBM_CUDA(cudaMemcpyAsync(&step0, da.state + 3, sizeof(double), cudaMemcpyDeviceToHost, s));
      GBM_CUDA(cudaStreamSynchronize(s));
      adapt_end = std::max<int64_t>(0, (int64_t)da.prm.num_adaptation_steps - (int64_t)step0);
    }
    r_free = std::min<int64_t>(num_results, std::max<int64_t>(0, adapt_end - burnin));
  }
  uint32_t t = first_step;
  for (int64_t r = 0; r < r_free; ++r) {
    const int64_t n = (r == 0) ? 1 + burnin : 1 + thin;
    for (int64_t i = 0; i < n; ++i, ++t) {
      NutsOutputs out{nq, nl, ng, b.lar, b.lf, b.acc, b.rmd, b.div, b.energy, nullptr};
      nuts_one_step(k, C, cq, cl, cg, eps, per_chain, step_key(seed, t), out);
      if (da.enabled)
        dual_averaging_update(s, b.lar, C, per_chain, da.prm, da.target_accept, da.state, eps);
      std::swap(cq, nq);
      std::swap(cl, nl);
      std::swap(cg, ng);
    }
    copy_row(tr.state ? tr.state + r * vec : nullptr, cq, vec, s);
    copy_row(tr.target_log_prob ? tr.target_log_prob + r * C : nullptr, cl, C, s);
    copy_row(tr.log_accept_ratio ? tr.log_accept_ratio + r * C : nullptr, b.lar, C, s);
    copy_row(tr.leapfrogs_taken ? tr.leapfrogs_taken + r * C : nullptr, b.lf, C, s);
    copy_row(tr.is_accepted ? tr.is_accepted + r * C : nullptr, b.acc, C, s);
    copy_row(tr.has_divergence ? tr.has_divergence + r * C : nullptr, b.div, C, s);
    copy_row(tr.step_size ? tr.step_size + r * groups : nullptr, eps, groups, s);
    moments_update(s, cq, vec, r, tr.moment_mean, tr.moment_m2);
  }
  if (r_free < num_results) {
    // Rows r_free .. num_results - 1 come from transitions burnin + r_free ..
    // of this call.  With r_free == 0 the burn-in transitions that precede
    // row 0 have not run yet: they run here, in lock-step.
    if (r_free == 0 && burnin > 0) {
      for (int64_t i = 0; i < burnin; ++i, ++t) {
        NutsOutputs out{nq, nl, ng, b.lar, b.lf, b.acc, b.rmd, b.div, b.energy, nullptr};
        nuts_one_step(k, C, cq, cl, cg, eps, per_chain, step_key(seed, t), out);
        if (da.enabled)
          dual_averaging_update(s, b.lar, C, per_chain, da.prm, da.target_accept, da.state, eps);
        std::swap(cq, nq);
        std::swap(cl, nl);
        std::swap(cg, ng);
      }
    }
    const int64_t K = num_results - r_free;
    double* lar = tr.log_accept_ratio ? tr.log_accept_ratio + r_free * C : nullptr;
    if (!lar && da.enabled) {   // the window counter and error sum follow every transition
      k->free_lar.reserve(sizeof(double) * (size_t)(K * C));
      lar = k->free_lar.as<double>();
    }
    FreeDev f{};
    f.tr_state = tr.state ? tr.state + r_free * vec : nullptr;
    f.tr_logp = tr.target_log_prob ? tr.target_log_prob + r_free * C : nullptr;
    f.tr_lar = lar;
    f.tr_lf = tr.leapfrogs_taken ? tr.leapfrogs_taken + r_free * C : nullptr;
    f.tr_acc = tr.is_accepted ? tr.is_accepted + r_free * C : nullptr;
    f.tr_div = tr.has_divergence ? tr.has_divergence + r_free * C : nullptr;
    f.tr_estride = vec;
    f.mom_mean = tr.moment_mean;
    f.mom_m2 = tr.moment_m2;
    f.mom_base = r_free;
    nuts_run_free(k, C, cq, cl, cg, eps, per_chain, seed, t, (int)K, INT64_MAX, f, nullptr);
    t += (uint32_t)K;
    // Each chain's last transition is its final state.
    const NutsDev& w = k->dev;
    copy_row(q, w.cand_q, vec, s);
    copy_row(g, w.cand_g, vec, s);
    copy_row(l, w.cand_l, C, s);
    cq = q;
    cl = l;
    cg = g;
    // Dual averaging past its window keeps the step size; its counter and
    // error sum advance with every transition's accept ratio, in order.
    for (int64_t r = 0; r < K; ++r) {
      if (da.enabled)
        dual_averaging_update(s, lar + r * C, C, per_chain, da.prm, da.target_accept, da.state,
                              eps);
      copy_row(tr.step_size ? tr.step_size + (r_free + r) * groups : nullptr, eps, groups, s);
    }
  }
  if (cq != q) {  // the final state lives in the scratch buffers: hand it back
    copy_row(q, cq, vec, s);
    copy_row(g, cg, vec, s);
    copy_row(l, cl, C, s);
  }
}

void hmc_sample_chain(gbm_hmc* k, int64_t C, float* q, double* l, float* g, float* eps,
                      int per_chain, int num_leapfrog_steps, uint2 seed, uint32_t first_step,
                      int64_t num_results, int64_t burnin, int64_t thin, const DaConfig& da,
                      const ChainTrace& tr) {
  cudaStream_t s = k->target->ctx->stream;
  const int64_t D = k->target->impl->dim;
  const size_t vec = (size_t)C * D;
  LoopBuffers b = carve(k->loop_mem, C, D);
  float *cq = q, *cg = g, *nq = b.q, *ng = b.g;
  double *cl = l, *nl = b.l;
  const int64_t groups = per_chain ? C : 1;
  // A transition is a fixed launch sequence: key from the device step
  // counter, the leapfrogs, the MH finish, dual averaging.  With graphs it is
  // captured once for each of the two ping-pong buffer assignments and
  // replayed for every step.
  uint2* keyp = k->key_dev.as<uint2>();
  uint32_t* stepp = reinterpret_cast<uint32_t*>(keyp + 1);
  set_step_kernel<<<1, 1, 0, s>>>(stepp, first_step);
  GBM_CUDA(cudaGetLastError());
  auto transition = [&](float* iq, double* il, float* ig, float* oq, double* ol, float* og,
                        cudaStream_t ls) {
    advance_step_key_kernel<<<1, 1, 0, ls>>>(seed, stepp, keyp);
    HmcOutputs out{oq, ol, og, nullptr, nullptr, nullptr, nullptr, nullptr,
                   b.corr, b.lar, b.acc};
    hmc_step_launches(k, C, iq, il, ig, eps, per_chain, num_leapfrog_steps, keyp, out, ls);
    if (da.enabled)
      dual_averaging_update(ls, b.lar, C, per_chain, da.prm, da.target_accept, da.state, eps);
  };
  cudaGraphExec_t graphs[2] = {nullptr, nullptr};
  cudaStream_t cs = nullptr;
  if (k->use_graphs) GBM_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  for (int64_t r = 0; r < num_results; ++r) {
    const int64_t n = (r == 0) ? 1 + burnin : 1 + thin;
    for (int64_t i = 0; i < n; ++i) {
      if (cs) {
        const int parity = cq == q ? 0 : 1;
        if (!graphs[parity]) {
          cudaGraph_t graph;
          GBM_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
          transition(cq, cl, cg, nq, nl, ng, cs);
          GBM_CUDA(cudaStreamEndCapture(cs, &graph));
          GBM_CUDA(cudaGraphInstantiate(&graphs[parity], graph, 0));
          GBM_CUDA(cudaGraphDestroy(graph));
        }
        GBM_CUDA(cudaGraphLaunch(graphs[parity], s));
      } else {
        transition(cq, cl, cg, nq, nl, ng, s);
      }
      std::swap(cq, nq);
      std::swap(cl, nl);
      std::swap(cg, ng);
    }
    copy_row(tr.state ? tr.state + r * vec : nullptr, cq, vec, s);
    copy_row(tr.target_log_prob ? tr.target_log_prob + r * C : nullptr, cl, C, s);
    copy_row(tr.log_accept_ratio ? tr.log_accept_ratio + r * C : nullptr, b.lar, C, s);
    copy_row(tr.is_accepted ? tr.is_accepted + r * C : nullptr, b.acc, C, s);
    copy_row(tr.step_size ? tr.step_size + r * groups : nullptr, eps, groups, s);
  }
  if (cq != q) {
    copy_row(q, cq, vec, s);
    copy_row(g, cg, vec, s);
    copy_row(l, cl, C, s);
  }
  if (cs) {
    GBM_CUDA(cudaStreamSynchronize(s));   // replays finished before the graphs go
    for (auto& gx : graphs)
      if (gx) cudaGraphExecDestroy(gx);
    cudaStreamDestroy(cs);
  }
}

}  // namespace gbm
