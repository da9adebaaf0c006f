// Internal C++ interfaces of the engine (not part of the C-ABI).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <memory>
#include <vector>

#include "common.cuh"

struct gbm_batch_member;   // include/gb300_mcmc.h

struct gbm_context {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool owns_stream = false;
  int num_sms = 0;
  // Pinned host words the host polls for NUTS loop control.
  int* host_flags = nullptr;
  int host_flag_slots = 0;
  // Error word in mapped pinned host memory: kernels whose bounded device
  // waits run out store a nonzero code through err_dev; the host reads
  // err_host without synchronizing (the store is visible once the kernel has
  // finished).
  volatile int* err_host = nullptr;
  int* err_dev = nullptr;
};

namespace gbm {

// Device memory owned by a handle; freed on destruction.
// Stream for stream-ordered allocation on this host thread (nullptr: plain
// cudaMalloc/cudaFree).  Job-server workers set it to their private stream so
// that creating and freeing a job's buffers never synchronizes the device.
cudaStream_t& alloc_stream();

struct DeviceBuffer {
  void* ptr = nullptr;
  size_t bytes = 0;
  cudaStream_t stream = nullptr;   // allocation stream (stream-ordered if set)
  DeviceBuffer() = default;
  DeviceBuffer(const DeviceBuffer&) = delete;
  DeviceBuffer& operator=(const DeviceBuffer&) = delete;
  ~DeviceBuffer() { release(); }
  void release() {
    if (ptr) {
      if (stream) cudaFreeAsync(ptr, stream); else cudaFree(ptr);
    }
    ptr = nullptr;
    bytes = 0;
  }
  void reserve(size_t b) {
    if (b <= bytes) return;
    release();
    if (b == 0) return;
    stream = alloc_stream();
    if (stream) {
      GBM_CUDA(cudaMallocAsync(&ptr, b, stream));
    } else {
      GBM_CUDA(cudaMalloc(&ptr, b));
    }
    bytes = b;
  }
  template <class T> T* as() const { return static_cast<T*>(ptr); }
};

// A built-in model family: batched log-density + gradient over a dense batch.
// Rows 0..n-1 of `q` (row stride ldq floats) are states; n is read on the
// device from *n_dev (so samplers can compact active chains without a host
// round trip) and never exceeds `cap`.  Outputs: logp[n] (float64),
// grad[n][ldg] (float32).  `ws` is scratch of workspace_bytes(cap).
struct Target {
  virtual ~Target() = default;
  int64_t dim = 0;
  virtual size_t workspace_bytes(int64_t cap) const = 0;
  virtual void eval(const float* q, int ldq, const int* n_dev, int cap, double* logp,
                    float* grad, int ldg, void* ws, cudaStream_t s) = 0;
  // Algorithmic flops and HBM bytes for one batched evaluation of n states.
  virtual double flops(int64_t n) const = 0;
  virtual double bytes(int64_t n) const = 0;
  // Kernels one eval() of up to `cap` states launches (launch accounting).
  virtual int launches_per_eval(int64_t cap) const = 0;
  // Ragged batches of posteriors (many targets of different dimension in one
  // sampler): per-chain element offsets and dimensions on the device, the
  // number of chains and the sum of their dimensions.  Uniform targets
  // return nullptr / 0.
  virtual const int64_t* ragged_offsets() const { return nullptr; }
  virtual const int* ragged_dims() const { return nullptr; }
  virtual int64_t ragged_chains() const { return 0; }
  virtual int64_t ragged_elements() const { return 0; }
  // Ragged evaluation in place: the chains act_idx[0 .. *act_count) (sorted),
  // states and gradients at their element offsets, logp indexed by chain.
  virtual void eval_active(const float* q, const int* act_idx, const int* act_count,
                           double* logp, float* grad, void* ws, cudaStream_t s) {}
};

// Fill / release a context (pinned host words, mapped error word).
void context_init(gbm_context* ctx, int device, cudaStream_t stream, bool owns_stream);
void context_free(gbm_context* ctx);
void set_error(const std::string& msg);

// Raise (and clear) an error a kernel stored in the context's error word.
inline void check_device_error(gbm_context* ctx) {
  const int e = ctx->err_host ? *ctx->err_host : 0;
  if (e) {
    *ctx->err_host = 0;
    throw DeviceTimeout{e};
  }
}

// Write the batch-size word `*count = n` on stream `s` (no host memory).
void set_count(int* count, int n, cudaStream_t s);

std::unique_ptr<Target> make_mvn(gbm_context* ctx, const float* loc, const float* scale_tril_inv,
                                 int64_t d, double log_norm);
std::unique_ptr<Target> make_hier(gbm_context* ctx, const float* y, const float* sigma, int64_t J,
                                  float mu_scale, float tau_scale);

std::unique_ptr<Target> make_batch(gbm_context* ctx, const ::gbm_batch_member* members,
                                   int64_t count);
// Chain tiles chosen by the batch autotuner (false: `t` is not a batch).
bool batch_schedule(const Target* t, int32_t* chain_tile);

std::unique_ptr<Target> make_transformed(gbm_context* ctx, Target* inner, const int32_t* codes);

// Any feature count, from library GEMMs (cuBLAS) and fused element-wise
// kernels: the FP32 target above 256 features, the mixed one above 512.
std::unique_ptr<Target> make_logreg_large(gbm_context* ctx, const void* X, int x_dtype, int64_t n,
                                          int64_t d, const float* y, float prior_scale,
                                          bool mixed);
// FP32 target for up to 128 features (row-pair layout, bulk-copied tiles);
// nullptr above that.
std::unique_ptr<Target> make_logreg_f32(gbm_context* ctx, const float* X, int64_t n, int64_t d,
                                        const float* y, float prior_scale);
std::unique_ptr<Target> make_logreg_simt(gbm_context* ctx, const float* X, int64_t n,
                                         int64_t d, const float* y, float prior_scale);

}  // namespace gbm

struct gbm_target {
  gbm_context* ctx = nullptr;
  std::unique_ptr<gbm::Target> impl;
  gbm::DeviceBuffer ws;       // eval scratch
  gbm::DeviceBuffer count;    // one int: batch size for direct calls
};
