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
// Keeps the reference's NaN for (-inf, -inf).  The sum is float64; the
// softplus term (argument <= 0, value in [0, ln 2]) is evaluated in float32,
// an absolute error of ~1e-7: a float64 exp/log1p pair is ~60 instructions
// on this GPU's narrow FP64 pipe, executed per chain per leaf.
__device__ __forceinline__ double log_add_exp(double x, double y) {
  double l = fmax(x, y);
  if (isnan(x) || isnan(y)) l = x + y;  // propagate NaN like tf.maximum
  const float d = (float)((x - l) + (y - l));
  return l + (double)log1pf(expf(d));
}

// log(1 - U) for a float32 uniform U in [0, 1), in float32 (see log_add_exp).
__device__ __forceinline__ double log1m_uniform(float U) { return (double)log1pf(-U); }

// e^x for x <= 0 over the whole float64 range (down to the subnormals) with
// float32 relative accuracy: e^x = 2^n 2^f with n = floor(x log2 e) applied
// exactly by ldexp and 2^f, f in [0, 1), from exp2f.  Used where a float32
// exponential would underflow (an acceptance probability e^-529 must still
// give log_accept_ratio -529) but a float64 exp costs too much.
__device__ __forceinline__ double exp_nonpositive(double x) {
  if (!(x > -746.0)) return x != x ? x : 0.0;   // NaN stays NaN; below the range: 0
  const double t = x * 1.4426950408889634;       // log2(e)
  const double n = floor(t);
  return ldexp((double)exp2f((float)(t - n)), (int)n);
}

}  // namespace gbm
