// A target seen through elementwise bijectors (TransformedTransitionKernel,
// mcmc/transformed_kernel.py:165-300, with make_transformed_log_prob,
// transformed_kernel.py:63-95): the sampler moves an unconstrained state x,
// the wrapped target is evaluated at y = f(x), and
//   log p~(x)      = log p(f(x)) + sum_d log |f_d'(x_d)|
//   grad log p~(x) = f'(x) * grad log p(f(x)) + d/dx sum_d log |f_d'(x_d)|.
// One bijector per state dimension, from the forward maps of
// bijectors/exp.py, softplus.py and sigmoid.py:
//   identity: f = x,              log f' = 0,                 (log f')' = 0
//   exp:      f = e^x,            log f' = x,                 (log f')' = 1
//   softplus: f = log(1 + e^x),   log f' = -softplus(-x),     (log f')' = sigmoid(-x)
//   sigmoid:  f = 1/(1 + e^-x),   log f' = -softplus(-x) - softplus(x),
//                                 (log f')' = 1 - 2 sigmoid(x)
// The log-Jacobian is summed in float64.
#include <cuda_runtime.h>

#include <memory>
#include <vector>

#include "engine.h"

namespace gbm {
namespace {

enum Bij : int8_t { kIdentity = 0, kExp = 1, kSoftplus = 2, kSigmoid = 3 };

__device__ __forceinline__ double softplus_d(double x) {
  return x > 0.0 ? x + log1p(exp(-x)) : log1p(exp(x));
}

__global__ void forward_kernel(const float* __restrict__ x, int ldx, const int* __restrict__ n_dev,
                               int D, const int8_t* __restrict__ code, float* __restrict__ y) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int n = *n_dev;
  if (i >= (size_t)n * D) return;
  const int c = (int)(i / D), d = (int)(i % D);
  const float v = x[(size_t)c * ldx + d];
  float out = v;
  switch (code[d]) {
    case kExp: out = expf(v); break;
    case kSoftplus: out = v > 0.f ? v + log1pf(expf(-v)) : log1pf(expf(v)); break;
    case kSigmoid: out = 1.f / (1.f + expf(-v)); break;
    default: break;
  }
  y[i] = out;
}

// One warp per chain: chain rule on the wrapped target's gradient and the
// log-Jacobian (float64 sum).
__global__ void jacobian_kernel(const float* __restrict__ x, int ldx, const int* __restrict__ n_dev,
                                int D, const int8_t* __restrict__ code,
                                const float* __restrict__ gy, double* __restrict__ logp,
                                float* __restrict__ grad, int ldg) {
  const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (c >= *n_dev) return;
  double ld = 0.0;
  for (int d = lane; d < D; d += 32) {
    const float v = x[(size_t)c * ldx + d];
    const float g = gy[(size_t)c * D + d];
    float out = g;
    switch (code[d]) {
      case kExp: {
        out = g * expf(v) + 1.f;
        ld += (double)v;
        break;
      }
      case kSoftplus: {
        const float sm = 1.f / (1.f + expf(v));        // sigmoid(-v) = f'(v) ... of -v
        const float s = 1.f - sm;                       // sigmoid(v) = f'(v)
        out = g * s + sm;
        ld -= softplus_d(-(double)v);
        break;
      }
      case kSigmoid: {
        const float s = 1.f / (1.f + expf(-v));
        out = g * s * (1.f - s) + (1.f - 2.f * s);
        ld -= softplus_d(-(double)v) + softplus_d((double)v);
        break;
      }
      default: break;
    }
    grad[(size_t)c * ldg + d] = out;
  }
  ld = warp_sum(ld);
  if (lane == 0) logp[c] += ld;
}

class Transformed final : public Target {
 public:
  Transformed(gbm_context* ctx, Target* inner, const int32_t* codes) : inner_(inner) {
    dim = inner->dim;
    std::vector<int8_t> h(dim);
    for (int64_t d = 0; d < dim; ++d) h[d] = (int8_t)codes[d];
    code_.reserve(dim);
    GBM_CUDA(cudaMemcpyAsync(code_.ptr, h.data(), dim, cudaMemcpyHostToDevice, ctx->stream));
    GBM_CUDA(cudaStreamSynchronize(ctx->stream));
  }

  size_t workspace_bytes(int64_t cap) const override {
    return 2 * align(sizeof(float) * (size_t)cap * dim) + inner_->workspace_bytes(cap);
  }

  void eval(const float* q, int ldq, const int* n_dev, int cap, double* logp, float* grad,
            int ldg, void* ws, cudaStream_t s) override {
    const int D = (int)dim;
    char* w = static_cast<char*>(ws);
    float* y = reinterpret_cast<float*>(w);
    float* gy = reinterpret_cast<float*>(w + align(sizeof(float) * (size_t)cap * D));
    void* inner_ws = w + 2 * align(sizeof(float) * (size_t)cap * D);
    const size_t total = (size_t)cap * D;
    forward_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(q, ldq, n_dev, D,
                                                                   code_.as<int8_t>(), y);
    GBM_CUDA(cudaGetLastError());
    inner_->eval(y, D, n_dev, cap, logp, gy, D, inner_ws, s);
    jacobian_kernel<<<(cap + 7) / 8, 256, 0, s>>>(q, ldq, n_dev, D, code_.as<int8_t>(), gy, logp,
                                                 grad, ldg);
    GBM_CUDA(cudaGetLastError());
  }

  int launches_per_eval(int64_t cap) const override {
    return inner_->launches_per_eval(cap) + 2;
  }
  double flops(int64_t n) const override { return inner_->flops(n) + 10.0 * (double)dim * n; }
  double bytes(int64_t n) const override { return inner_->bytes(n) + 16.0 * (double)dim * n; }

 private:
  static size_t align(size_t b) { return (b + 255) / 256 * 256; }
  Target* inner_;
  DeviceBuffer code_;
};

}  // namespace

std::unique_ptr<Target> make_transformed(gbm_context* ctx, Target* inner, const int32_t* codes) {
  return std::unique_ptr<Target>(new Transformed(ctx, inner, codes));
}

}  // namespace gbm
