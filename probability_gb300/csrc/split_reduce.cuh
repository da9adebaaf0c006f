// Deterministic sum of per-split partial results of a row-split logistic
// regression evaluation, plus the Normal(0, s) prior.
//
// Layout written by the partial kernels: lpart[S][n] (float64) and
// gpart[S][n][D] (float32), where S = number of row splits for n chains:
//   S = clamp(grid / ceil(n / ct), 1, ceil(N / nt)).
// One warp per chain: each lane owns features lane + 32k (D <= DMAX) and adds
// the splits in index order, U splits' loads in flight at a time; the
// log-density terms (likelihood partials, prior, linear part) are combined
// per lane and summed by one float64 warp reduction.  The order depends only
// on S and D, so results are reproducible.
//
// `lin` (optional, float64 [D]) adds lin . q_c to each chain's log-density:
// the tensor-core kernels leave the linear part sum_r (y_r - 1/2) z_rc of the
// Bernoulli log-likelihood to this pass as (X^T (y - 1/2)) . q_c, exact in
// float64.
#pragma once
#include <cuda_runtime.h>

#include "common.cuh"

namespace gbm {

constexpr int kReduceWarps = 4;            // chains per CTA

// Chains of one launch.  A launch covers at most grid * ct chains (one work
// item per CTA); larger batches are evaluated as consecutive chunks of
// `c_lim` chains starting at chain `c_base` (pointers offset by the caller).
// Chunk k sees min(max(n - c_base, 0), c_lim) chains of the n in *n_dev.
__host__ __device__ __forceinline__ int chunk_count(int n, int c_base, int c_lim) {
  const int m = n - c_base;
  return m < 0 ? 0 : (m > c_lim ? c_lim : m);
}

// CTAs (or CTA pairs) of one launch: at most grid_max, and no more than the
// call's chain tiles times the row splits that keep at least min_rows rows
// each, so no CTA is launched only to find no work.  With min_rows = 64 (the
// smallest row tile) the split counts are those of the full grid: a small,
// latency-bound evaluation keeps one row tile per CTA.  Kernels and the split
// reduction derive the split count from the grid they are given, so passing
// this value to both keeps them consistent.
inline int work_grid(int grid_max, int64_t chains, int ct, int64_t N, int64_t min_rows) {
  const int64_t tiles = (chains + ct - 1) / ct;
  const int64_t s_cap = N / min_rows > 1 ? N / min_rows : 1;
  int64_t g = tiles * s_cap;
  if (g > grid_max) g = grid_max;
  return g < 1 ? 1 : (int)g;
}

constexpr int64_t kMinSplitRows = 64;

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
                    const float* __restrict__ Q, int ldq, const int* __restrict__ n_dev,
                    int c_base, int c_lim, int ct, int nt, int grid, int N, int D,
                    float inv_var, double log_norm, const double* __restrict__ lin,
                    double* __restrict__ logp, float* __restrict__ grad, int ldg) {
  constexpr int kK = DMAX / 32;               // features per lane
  constexpr int U = DMAX <= 128 ? 8 : 4;      // splits in flight
  const int n = chunk_count(*n_dev, c_base, c_lim);
  const int c = blockIdx.x * kReduceWarps + (threadIdx.x >> 5);
  if (c >= n) return;
  const int lane = threadIdx.x & 31;
  const int S = split_count(n, ct, nt, grid, N);
  const size_t sstride = (size_t)n * D;
  const float* p = gpart + (size_t)c * D;
  float acc[kK];
#pragma unroll
  for (int k = 0; k < kK; ++k) acc[k] = 0.f;
  int s = 0;
  for (; s + U <= S; s += U) {
    float v[U][kK];
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int k = 0; k < kK; ++k) {
        const int d = lane + 32 * k;
        v[u][k] = d < D ? p[(size_t)(s + u) * sstride + d] : 0.f;
      }
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int k = 0; k < kK; ++k) acc[k] += v[u][k];
  }
  for (; s < S; ++s)
#pragma unroll
    for (int k = 0; k < kK; ++k) {
      const int d = lane + 32 * k;
      if (d < D) acc[k] += p[(size_t)s * sstride + d];
    }
  // Per-lane log-density terms: likelihood partials of splits lane, lane + 32,
  // ..., then lin . q - q.q / (2 s^2) over this lane's features.
  double t = 0.0;
  for (int j = lane; j < S; j += 32) t += lpart[(size_t)j * n + c];
  double pr = 0.0, li = 0.0;
#pragma unroll
  for (int k = 0; k < kK; ++k) {
    const int d = lane + 32 * k;
    if (d < D) {
      const float q = Q[(size_t)c * ldq + d];
      const double qd = (double)q;
      pr += qd * qd;
      if (lin) li += lin[d] * qd;
      grad[(size_t)c * ldg + d] = acc[k] - q * inv_var;
    }
  }
  t = warp_sum(t + li - 0.5 * (double)inv_var * pr);
  if (lane == 0) logp[c] = t + (double)D * log_norm;
}

// Q, logp and grad point at chain c_base of the batch; `cap` bounds this
// chunk's chains (<= c_lim).
void launch_split_reduce(const double* lpart, const float* gpart, const float* Q, int ldq,
                         const int* n_dev, int c_base, int c_lim, int cap, int ct, int nt,
                         int grid, int N, int D, float inv_var, double log_norm,
                         const double* lin, double* logp, float* grad, int ldg, cudaStream_t s) {
  const unsigned blocks = (unsigned)((cap + kReduceWarps - 1) / kReduceWarps);
  if (D <= 128)
    split_reduce_kernel<128><<<blocks, 32 * kReduceWarps, 0, s>>>(
        lpart, gpart, Q, ldq, n_dev, c_base, c_lim, ct, nt, grid, N, D, inv_var, log_norm, lin,
        logp, grad, ldg);
  else if (D <= 256)
    split_reduce_kernel<256><<<blocks, 32 * kReduceWarps, 0, s>>>(
        lpart, gpart, Q, ldq, n_dev, c_base, c_lim, ct, nt, grid, N, D, inv_var, log_norm, lin,
        logp, grad, ldg);
  else
    split_reduce_kernel<512><<<blocks, 32 * kReduceWarps, 0, s>>>(
        lpart, gpart, Q, ldq, n_dev, c_base, c_lim, ct, nt, grid, N, D, inv_var, log_norm, lin,
        logp, grad, ldg);
  GBM_CUDA(cudaGetLastError());
}

}  // namespace

}  // namespace gbm
