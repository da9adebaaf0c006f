// Shared device/host helpers for the gb300 MCMC engine (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <string>

namespace gbm {

// Status codes returned by every C-ABI entry point (see include/gb300_mcmc.h).
enum Status : int {
  kOk = 0,
  kInvalid = 22,     // EINVAL: shapes, dtypes, configuration
  kNoMemory = 12,    // ENOMEM: device allocation or memory budget
  kNotSupported = 95,
  kTimedOut = 110,   // ETIMEDOUT: a bounded device wait ran out
  kCuda = 1000,      // a CUDA runtime error (message in gbm_last_error)
};

void set_error(const std::string& msg);

struct CudaError {
  cudaError_t err;
  const char* what;
};

// A kernel's bounded device wait ran out; `code` says which wait.
struct DeviceTimeout {
  int code;
};

#define GBM_CUDA(call)                                                     \
  do {                                                                     \
    cudaError_t _e = (call);                                               \
    if (_e != cudaSuccess) throw ::gbm::CudaError{_e, #call};              \
  } while (0)

constexpr int kWarp = 32;

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// softplus(x) = log(1 + exp(x)), stable for both tails.
__device__ __forceinline__ float softplusf(float x) {
  return fmaxf(x, 0.f) + log1pf(expf(-fabsf(x)));
}

__device__ __forceinline__ double softplus_d(double x) {
  return fmax(x, 0.0) + log1p(exp(-fabs(x)));
}

// math/generic.py:585-612 log_add_exp: larger + softplus((x-l) + (y-l)).
// Keeps the reference's NaN for (-inf, -inf).
__device__ __forceinline__ double log_add_exp(double x, double y) {
  double l = fmax(x, y);
  if (isnan(x) || isnan(y)) l = x + y;  // propagate NaN like tf.maximum
  return l + softplus_d((x - l) + (y - l));
}

}  // namespace gbm
