// Deterministic sum of per-split partial results of a row-split logistic
// regression evaluation, plus the Normal(0, s) prior.
//
// Layout written by the partial kernels: lpart[S][n] (float64) and
// gpart[S][n][D] (float32), where S = number of row splits for n chains:
//   S = clamp(grid / ceil(n / ct), 1, ceil(N / nt)).
// One CTA per chain: warp w sums splits w, w + W, w + 2W, ... (each lane
// owns features lane + 32k, D <= 512), then the W partial sums are combined
// in warp order.  The order depends only on S, so results are reproducible;
// with many splits (few chains) all W warps keep loads in flight.
//
// `lin` (optional, float64 [D]) adds lin . q_c to each chain's log-density:
// the tensor-core kernel leaves the linear part sum_r (y_r - 1/2) z_rc of the
// Bernoulli log-likelihood to this pass as (X^T (y - 1/2)) . q_c, exact in
// float64.
#pragma once
#include <cuda_runtime.h>

#include "common.cuh"

namespace gbm {

constexpr int kReduceWarps = 8;

namespace {

__device__ __forceinline__ int split_count(int n, int ct, int nt, int grid, int N) {
  const int tiles = (n + ct - 1) / ct;
  if (tiles == 0) return 0;
  int s = grid / tiles;
  s = s < 1 ? 1 : s;
  const int row_tiles = (N + nt - 1) / nt;
  return s > row_tiles ? row_tiles : s;
}

template <int DMAX>
__global__ void __launch_bounds__(32 * kReduceWarps)
split_reduce_kernel(const double* __restrict__ lpart, const float* __restrict__ gpart,
                    const float* __restrict__ Q, int ldq, const int* __restrict__ n_dev, int ct,
                    int nt, int grid, int N, int D, float inv_var, double log_norm,
                    const double* __restrict__ lin, double* __restrict__ logp,
                    float* __restrict__ grad, int ldg) {
  const int n = *n_dev;
  const int c = blockIdx.x;
  if (c >= n) return;
  const int S = split_count(n, ct, nt, grid, N);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __shared__ float gsum[kReduceWarps][DMAX];
  __shared__ double lsum[kReduceWarps];
  __shared__ double prior_s;
  const size_t sstride = (size_t)n * D;
  const float* p = gpart + (size_t)c * D;
  constexpr int kK = DMAX / 32;
  float acc[kK];
#pragma unroll
  for (int k = 0; k < kK; ++k) acc[k] = 0.f;
  double lp = 0.0;
  // Four splits' loads in flight per warp step (same summation order).
  int s = warp;
  for (; s + 3 * kReduceWarps < S; s += 4 * kReduceWarps) {
    float v[4][kK];
    double l4[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const size_t base = (size_t)(s + u * kReduceWarps) * sstride;
#pragma unroll
      for (int k = 0; k < kK; ++k) {
        const int d = lane + 32 * k;
        v[u][k] = d < D ? p[base + d] : 0.f;
      }
      l4[u] = lane == 0 ? lpart[(size_t)(s + u * kReduceWarps) * n + c] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
#pragma unroll
      for (int k = 0; k < kK; ++k) acc[k] += v[u][k];
      lp += l4[u];
    }
  }
  for (; s < S; s += kReduceWarps) {
#pragma unroll
    for (int k = 0; k < kK; ++k) {
      const int d = lane + 32 * k;
      if (d < D) acc[k] += p[(size_t)s * sstride + d];
    }
    if (lane == 0) lp += lpart[(size_t)s * n + c];
  }
#pragma unroll
  for (int k = 0; k < kK; ++k) gsum[warp][lane + 32 * k] = acc[k];
  if (lane == 0) lsum[warp] = lp;
  if (warp == 0) {
    double pr = 0.0, li = 0.0;
    for (int d = lane; d < D; d += 32) {
      const double qd = (double)Q[(size_t)c * ldq + d];
      pr += qd * qd;
      if (lin) li += lin[d] * qd;
    }
    pr = warp_sum(pr);
    li = warp_sum(li);
    if (lane == 0) prior_s = li - 0.5 * (double)inv_var * pr;
  }
  __syncthreads();
  for (int d = threadIdx.x; d < D; d += 32 * kReduceWarps) {
    float t = 0.f;
#pragma unroll
    for (int w = 0; w < kReduceWarps; ++w) t += gsum[w][d];
    grad[(size_t)c * ldg + d] = t - Q[(size_t)c * ldq + d] * inv_var;
  }
  if (threadIdx.x == 0) {
    double t = 0.0;
#pragma unroll
    for (int w = 0; w < kReduceWarps; ++w) t += lsum[w];
    logp[c] = t + prior_s + (double)D * log_norm;
  }
}

void launch_split_reduce(const double* lpart, const float* gpart, const float* Q, int ldq,
                         const int* n_dev, int cap, int ct, int nt, int grid, int N, int D,
                         float inv_var, double log_norm, const double* lin, double* logp,
                         float* grad, int ldg, cudaStream_t s) {
  if (D <= 256)
    split_reduce_kernel<256><<<cap, 32 * kReduceWarps, 0, s>>>(
        lpart, gpart, Q, ldq, n_dev, ct, nt, grid, N, D, inv_var, log_norm, lin, logp, grad, ldg);
  else
    split_reduce_kernel<512><<<cap, 32 * kReduceWarps, 0, s>>>(
        lpart, gpart, Q, ldq, n_dev, ct, nt, grid, N, D, inv_var, log_norm, lin, logp, grad, ldg);
  GBM_CUDA(cudaGetLastError());
}

}  // namespace

}  // namespace gbm
