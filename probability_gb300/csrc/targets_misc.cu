// Multivariate-normal and non-centred hierarchical-normal targets.
//
// MultivariateNormalTriL (distributions/mvn_tril.py:44, log_prob through
// mvn_linear_operator.py:242, which solves with the scale factor L):
//   u = L^-1 (x - mu),  logp = -1/2 |u|^2 + log_norm,  grad = -L^-T u
// with L^-1 and log_norm = -sum log|L_ii| - D/2 log 2pi supplied by the
// caller (computed once from scale_tril).  Working with L^-1 keeps the
// conditioning of L (the square root of the covariance's) -- multiplying by
// the precision L^-T L^-1 in FP32 would square it.  Both products are
// register-tiled triangular GEMMs over all chains on the CUDA cores; each CTA
// of the first also forms its slice of |u|^2 and a third kernel sums the
// slices in fixed order (deterministic).
//
// Non-centred hierarchical normal, the eight-schools pattern of
// mcmc/eight_schools_hmc.py:41-58 with mu ~ N(0, s_mu), tau ~ HalfCauchy(0,
// s_tau) (distributions/half_cauchy.py:138-145) sampled as log tau with its
// log-Jacobian, z_j ~ N(0, 1), y_j ~ N(mu + tau z_j, sigma_j).  State =
// [mu, log tau, z_1..z_J]; one warp per chain.
#include <cuda_runtime.h>

#include <memory>

#include "engine.h"

namespace gbm {
namespace {

constexpr int kTile = 64;     // chains x features per CTA tile
constexpr int kKc = 32;       // K chunk
constexpr int kMvnThreads = 256;

// Two triangular GEMMs over all chains with M = L^-1 (lower triangular):
//   MODE 0:  U[c][i] = sum_{k <= i} (Q[c][k] - mu[k]) M[i][k],
//            part[c][itile] = sum_{i in tile} U[c][i]^2
//   MODE 1:  G[c][j] = -sum_{i >= j} U[c][i] M[i][j]
// K-chunks that lie entirely in the zero triangle are skipped.
template <int MODE>
__global__ void __launch_bounds__(kMvnThreads)
mvn_tri_kernel(const float* __restrict__ A, int lda, const int* __restrict__ n_dev, int D,
               const float* __restrict__ mu, const float* __restrict__ M,
               float* __restrict__ out, int ldo, double* __restrict__ part, int dtiles) {
  const int n = *n_dev;
  const int c0 = blockIdx.y * kTile, o0 = blockIdx.x * kTile;
  if (c0 >= n) return;
  __shared__ float As[kKc][kTile + 4];   // [k][chain]
  __shared__ float Bs[kKc][kTile + 4];   // [k][output column]
  __shared__ double red[16][kTile];
  const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
  float acc[4][4] = {};
  const int k_begin = MODE == 0 ? 0 : (o0 / kKc) * kKc;
  const int k_end = MODE == 0 ? min(D, o0 + kTile) : D;
  for (int k0 = k_begin; k0 < k_end; k0 += kKc) {
    for (int i = tid; i < kKc * kTile; i += kMvnThreads) {
      const int kk = i % kKc, cc = i / kKc;
      const int c = c0 + cc, k = k0 + kk;
      float a = 0.f;
      if (c < n && k < D) a = MODE == 0 ? A[(size_t)c * lda + k] - mu[k] : A[(size_t)c * lda + k];
      As[kk][cc] = a;
      if (MODE == 0) {        // B(k, i) = M[i][k]: k contiguous in memory
        const int oo = i / kKc, o = o0 + oo;
        Bs[kk][oo] = (o < D && k < D && k <= o) ? M[(size_t)o * D + k] : 0.f;
      } else {                // B(i, j) = M[i][j]: j contiguous in memory
        const int oo = i % kTile, kr = i / kTile;
        const int o = o0 + oo, k2 = k0 + kr;
        Bs[kr][oo] = (o < D && k2 < D && k2 >= o) ? M[(size_t)k2 * D + o] : 0.f;
      }
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < kKc; ++kk) {
      const float4 a4 = *reinterpret_cast<const float4*>(&As[kk][ty * 4]);
      const float4 b4 = *reinterpret_cast<const float4*>(&Bs[kk][tx * 4]);
      const float aa[4] = {a4.x, a4.y, a4.z, a4.w};
      const float bb[4] = {b4.x, b4.y, b4.z, b4.w};
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(aa[i], bb[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int c = c0 + ty * 4 + i;
    double sq = 0.0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int o = o0 + tx * 4 + j;
      if (c < n && o < D) {
        const float v = MODE == 0 ? acc[i][j] : -acc[i][j];
        out[(size_t)c * ldo + o] = v;
        sq += (double)v * (double)v;
      }
    }
    if (MODE == 0) red[tx][ty * 4 + i] = sq;
  }
  if (MODE == 0) {
    __syncthreads();
    if (tid < kTile && c0 + tid < n) {
      double s = 0.0;
      for (int t = 0; t < 16; ++t) s += red[t][tid];
      part[(size_t)(c0 + tid) * dtiles + blockIdx.x] = s;
    }
  }
}

__global__ void mvn_finish_kernel(const double* __restrict__ part, int dtiles,
                                  const int* __restrict__ n_dev, double log_norm,
                                  double* __restrict__ logp) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= *n_dev) return;
  double s = 0.0;
  for (int t = 0; t < dtiles; ++t) s += part[(size_t)c * dtiles + t];
  logp[c] = -0.5 * s + log_norm;   // -1/2 |L^-1 (x - mu)|^2
}

class Mvn final : public Target {
 public:
  Mvn(gbm_context* ctx, const float* loc, const float* scale_tril_inv, int64_t d, double log_norm)
      : log_norm_(log_norm) {
    dim = d;
    mu_.reserve(sizeof(float) * d);
    m_.reserve(sizeof(float) * d * d);
    GBM_CUDA(cudaMemcpyAsync(mu_.ptr, loc, sizeof(float) * d, cudaMemcpyDeviceToDevice,
                             ctx->stream));
    GBM_CUDA(cudaMemcpyAsync(m_.ptr, scale_tril_inv, sizeof(float) * d * d,
                             cudaMemcpyDeviceToDevice, ctx->stream));
    dtiles_ = (int)((d + kTile - 1) / kTile);
  }
  size_t workspace_bytes(int64_t cap) const override {
    return sizeof(double) * (size_t)cap * dtiles_ + sizeof(float) * (size_t)cap * dim + 512;
  }
  void eval(const float* q, int ldq, const int* n_dev, int cap, double* logp, float* grad,
            int ldg, void* ws, cudaStream_t s) override {
    double* part = static_cast<double*>(ws);
    float* u = reinterpret_cast<float*>(part + (size_t)cap * dtiles_);
    dim3 grid(dtiles_, (cap + kTile - 1) / kTile);
    const int D = (int)dim;
    mvn_tri_kernel<0><<<grid, kMvnThreads, 0, s>>>(q, ldq, n_dev, D, mu_.as<float>(),
                                                   m_.as<float>(), u, D, part, dtiles_);
    mvn_tri_kernel<1><<<grid, kMvnThreads, 0, s>>>(u, D, n_dev, D, mu_.as<float>(),
                                                   m_.as<float>(), grad, ldg, part, dtiles_);
    GBM_CUDA(cudaGetLastError());
    mvn_finish_kernel<<<(cap + 255) / 256, 256, 0, s>>>(part, dtiles_, n_dev, log_norm_, logp);
    GBM_CUDA(cudaGetLastError());
  }
  int launches_per_eval(int64_t) const override { return 3; }
  // Two triangular GEMMs: ~D^2 multiply-adds each per chain.
  double flops(int64_t n) const override { return 2.0 * (double)dim * dim * n; }
  double bytes(int64_t n) const override {
    return 4.0 * (double)dim * dim + 8.0 * (double)n * dim + 8.0 * n;
  }

 private:
  double log_norm_;
  int dtiles_ = 1;
  DeviceBuffer mu_, m_;
};

// ---------------------------------------------------------------------------
__global__ void hier_kernel(const float* __restrict__ Q, int ldq, const int* __restrict__ n_dev,
                            int J, const float* __restrict__ y, const float* __restrict__ sigma,
                            float mu_scale, float tau_scale, double const_term,
                            double* __restrict__ logp, float* __restrict__ G, int ldg) {
  const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (c >= *n_dev) return;
  const float* x = Q + (size_t)c * ldq;
  const float mu = x[0], eta = x[1];
  const float tau = expf(eta);
  float lp = 0.f, gmu = 0.f, geta = 0.f;
  for (int j = lane; j < J; j += 32) {
    const float z = x[2 + j];
    const float s = sigma[j];
    const float res = (y[j] - (mu + tau * z)) / s;    // standardized residual
    const float r = res / s;                           // d/dtheta log N(y; theta, s)
    lp += -0.5f * z * z - 0.5f * res * res;
    gmu += r;
    geta += r * z;
    G[(size_t)c * ldg + 2 + j] = -z + tau * r;
  }
  double lpd = warp_sum((double)lp);
  gmu = warp_sum(gmu);
  geta = warp_sum(geta);
  if (lane == 0) {
    const float t = tau / tau_scale;
    // priors: mu ~ N(0, s_mu); tau ~ HalfCauchy(0, s_tau) with log-Jacobian eta
    lpd += -0.5 * (double)(mu / mu_scale) * (double)(mu / mu_scale) - log1p((double)t * t) +
           (double)eta + const_term;
    logp[c] = lpd;
    G[(size_t)c * ldg + 0] = -mu / (mu_scale * mu_scale) + gmu;
    G[(size_t)c * ldg + 1] = -2.f * t * t / (1.f + t * t) + 1.f + tau * geta;
  }
}

class Hier final : public Target {
 public:
  Hier(gbm_context* ctx, const float* y, const float* sigma, int64_t J, float mu_scale,
       float tau_scale, double const_term)
      : J_(J), mu_scale_(mu_scale), tau_scale_(tau_scale), const_(const_term) {
    dim = J + 2;
    y_.reserve(sizeof(float) * J);
    s_.reserve(sizeof(float) * J);
    GBM_CUDA(cudaMemcpyAsync(y_.ptr, y, sizeof(float) * J, cudaMemcpyDeviceToDevice, ctx->stream));
    GBM_CUDA(cudaMemcpyAsync(s_.ptr, sigma, sizeof(float) * J, cudaMemcpyDeviceToDevice,
                             ctx->stream));
  }
  size_t workspace_bytes(int64_t) const override { return 256; }
  void eval(const float* q, int ldq, const int* n_dev, int cap, double* logp, float* grad,
            int ldg, void*, cudaStream_t s) override {
    hier_kernel<<<(cap + 7) / 8, 256, 0, s>>>(q, ldq, n_dev, (int)J_, y_.as<float>(),
                                              s_.as<float>(), mu_scale_, tau_scale_, const_,
                                              logp, grad, ldg);
    GBM_CUDA(cudaGetLastError());
  }
  int launches_per_eval(int64_t) const override { return 1; }
  double flops(int64_t n) const override { return 10.0 * (double)J_ * n; }
  double bytes(int64_t n) const override { return 8.0 * J_ + 8.0 * (double)(J_ + 2) * n + 8.0 * n; }

 private:
  int64_t J_;
  float mu_scale_, tau_scale_;
  double const_;
  DeviceBuffer y_, s_;
};

}  // namespace

std::unique_ptr<Target> make_mvn(gbm_context* ctx, const float* loc, const float* scale_tril_inv,
                                 int64_t d, double log_norm) {
  return std::unique_ptr<Target>(new Mvn(ctx, loc, scale_tril_inv, d, log_norm));
}

std::unique_ptr<Target> make_hier(gbm_context* ctx, const float* y, const float* sigma, int64_t J,
                                  float mu_scale, float tau_scale) {
  // Constant part of the log-density: HalfCauchy and Normal normalizers.
  std::unique_ptr<float[]> hs(new float[J]);
  GBM_CUDA(cudaMemcpyAsync(hs.get(), sigma, sizeof(float) * J, cudaMemcpyDeviceToHost,
                           ctx->stream));
  GBM_CUDA(cudaStreamSynchronize(ctx->stream));
  const double log2pi = log(2.0 * M_PI);
  double c = log(2.0 / M_PI) - log((double)mu_scale) - log((double)tau_scale) -
             0.5 * (1.0 + 2.0 * (double)J) * log2pi;
  for (int64_t j = 0; j < J; ++j) c -= log((double)hs[j]);
  return std::unique_ptr<Target>(new Hier(ctx, y, sigma, J, mu_scale, tau_scale, c));
}

}  // namespace gbm
