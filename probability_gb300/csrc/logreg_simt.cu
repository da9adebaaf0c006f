// Fused logistic-regression log-density + gradient, FP32 CUDA cores.
//
// For a dense batch of n chain states B[n][D] and data X[N][D], y[N]:
//   z      = X B^T                           (N x n)
//   logp_c = sum_r [-softplus(z) (1-y) - softplus(-z) y] + log N(B_c; 0, s)
//   R      = y - sigmoid(z)
//   grad_c = X^T R_c - B_c / s^2
// which is what the reference obtains by autodiff of the inference_gym
// logistic-regression target (spinoffs/inference_gym/inference_gym/targets/
// logistic_regression.py:92-103 with distributions/bernoulli.py:126-140).
//
// One CTA owns a (chain tile of 64, row split) work item.  Per 64-row tile of
// X it computes Z = X_tile B_tile^T (register-tiled 4x4 per thread), the
// log-likelihood and R in the epilogue (R goes to shared memory only), then
// G += R^T X_tile with G held in registers across the CTA's rows: X is read
// from HBM/L2 once per chain tile and Z/R never leave the SM.  Each CTA
// writes one partial (logp, G); a second kernel sums the partials in fixed
// split order (deterministic) and adds the prior.
#include <cuda_runtime.h>

#include <algorithm>
#include <memory>

#include "engine.h"
#include "split_reduce.cuh"

namespace gbm {

constexpr int kCT = 64;        // chains per tile
constexpr int kNT = 64;        // data rows per tile
constexpr int kThreads = 256;
constexpr int kXPad = kNT + 4;  // Xt row stride (floats)

__host__ __device__ inline int num_splits(int n, int grid, int row_tiles) {
  const int tiles = (n + kCT - 1) / kCT;
  if (tiles == 0) return 0;
  int s = grid / tiles;
  s = s < 1 ? 1 : s;
  return s > row_tiles ? row_tiles : s;
}

__device__ __forceinline__ float sigmoidf_(float z) { return 1.f / (1.f + expf(-z)); }

template <int KD>
__global__ void __launch_bounds__(kThreads)
logreg_partial_kernel(const float* __restrict__ X, int ldx, const float* __restrict__ y, int N,
                      int D, const float* __restrict__ Q, int ldq, const int* __restrict__ n_dev,
                      int c_base, int c_lim, int grid, double* __restrict__ lpart,
                      float* __restrict__ gpart) {
  extern __shared__ __align__(16) float smem[];
  const int n = chunk_count(*n_dev, c_base, c_lim);
  const int row_tiles = (N + kNT - 1) / kNT;
  const int S = num_splits(n, grid, row_tiles);
  const int tiles = (n + kCT - 1) / kCT;
  const int item = blockIdx.x;
  if (S == 0 || item >= tiles * S) return;
  const int tile = item % tiles, split = item / tiles;
  const int c0 = tile * kCT;
  const int rt_begin = (int)((long long)split * row_tiles / S);
  const int rt_end = (int)((long long)(split + 1) * row_tiles / S);
  const int Dp = KD * 16;  // padded feature count held in shared memory

  float* Bt = smem;                    // [Dp][kCT]
  float* Xt = Bt + Dp * kCT;           // [Dp][kXPad]
  float* Rs = Xt + Dp * kXPad;         // [kNT][kCT]
  __shared__ double red[kThreads / 16][16][4];

  const int tid = threadIdx.x;
  // B tile, transposed: Bt[d][c] = Q[c0 + c][d]; zero outside (n, D).
  for (int i = tid; i < Dp * kCT; i += kThreads) {
    const int c = i / Dp, d = i % Dp;
    float v = 0.f;
    if (c0 + c < n && d < D) v = Q[(size_t)(c0 + c) * ldq + d];
    Bt[d * kCT + c] = v;
  }
  // Rows of Xt beyond D stay zero for the whole kernel.
  for (int i = tid; i < (Dp - D) * kXPad; i += kThreads) Xt[D * kXPad + i] = 0.f;

  const int ty = tid >> 4, tx = tid & 15;   // phase 1: rows ty*4.., chains tx*4..
  const int cg = tid >> 4, dg = tid & 15;   // phase 2: chains cg*4.., d = dg + 16k
  float g[4][KD];
#pragma unroll
  for (int j = 0; j < 4; ++j)
#pragma unroll
    for (int k = 0; k < KD; ++k) g[j][k] = 0.f;
  double lp_acc[4] = {0.0, 0.0, 0.0, 0.0};

  for (int rt = rt_begin; rt < rt_end; ++rt) {
    const int r0 = rt * kNT;
    __syncthreads();  // previous tile's phase 2 is done with Xt/Rs
    // X tile, transposed into Xt[d][r] (coalesced global reads along d).
    for (int i = tid; i < kNT * D; i += kThreads) {
      const int r = i / D, d = i % D;
      const int row = r0 + r;
      Xt[d * kXPad + r] = row < N ? X[(size_t)row * ldx + d] : 0.f;
    }
    __syncthreads();
    // Phase 1: Z[r][c] = sum_d Xt[d][r] Bt[d][c].
    float acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
    for (int d = 0; d < D; ++d) {
      const float4 xv = *reinterpret_cast<const float4*>(&Xt[d * kXPad + ty * 4]);
      const float4 bv = *reinterpret_cast<const float4*>(&Bt[d * kCT + tx * 4]);
      const float xa[4] = {xv.x, xv.y, xv.z, xv.w};
      const float ba[4] = {bv.x, bv.y, bv.z, bv.w};
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(xa[i], ba[j], acc[i][j]);
    }
    // Epilogue: log-likelihood terms and residuals R = y - sigmoid(z).
    float lp_tile[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int row = r0 + ty * 4 + i;
      const bool ok = row < N;
      const float yv = ok ? y[row] : 0.f;
      float rv[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const float z = acc[i][j];
        // bernoulli.py:126-140: -softplus(z) (1 - y) - softplus(-z) y
        const float lp = -softplusf(z) * (1.f - yv) - softplusf(-z) * yv;
        lp_tile[j] += ok ? lp : 0.f;
        rv[j] = ok ? (yv - sigmoidf_(z)) : 0.f;
      }
      *reinterpret_cast<float4*>(&Rs[(ty * 4 + i) * kCT + tx * 4]) =
          make_float4(rv[0], rv[1], rv[2], rv[3]);
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) lp_acc[j] += (double)lp_tile[j];
    __syncthreads();
    // Phase 2: G[c][d] += sum_r Rs[r][c] Xt[d][r].
    for (int r = 0; r < kNT; ++r) {
      const float4 rv4 = *reinterpret_cast<const float4*>(&Rs[r * kCT + cg * 4]);
      const float ra[4] = {rv4.x, rv4.y, rv4.z, rv4.w};
#pragma unroll
      for (int k = 0; k < KD; ++k) {
        const float xv = Xt[(dg + 16 * k) * kXPad + r];
#pragma unroll
        for (int j = 0; j < 4; ++j) g[j][k] = fmaf(ra[j], xv, g[j][k]);
      }
    }
  }

  // Partial log-likelihood: reduce the 16 row groups (ty) of each chain.
#pragma unroll
  for (int j = 0; j < 4; ++j) red[ty][tx][j] = lp_acc[j];
  __syncthreads();
  if (tid < kCT) {
    const int c = tid;
    double s = 0.0;
    for (int t = 0; t < kThreads / 16; ++t) s += red[t][c >> 2][c & 3];
    if (c0 + c < n) lpart[(size_t)split * n + c0 + c] = s;
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int c = c0 + cg * 4 + j;
    if (c >= n) continue;
    float* dst = gpart + ((size_t)split * n + c) * D;
#pragma unroll
    for (int k = 0; k < KD; ++k) {
      const int d = dg + 16 * k;
      if (d < D) dst[d] = g[j][k];
    }
  }
}

// One warp per state: sum the split partials in fixed order, add the prior.
__global__ void logreg_reduce_kernel(const double* __restrict__ lpart,
                                     const float* __restrict__ gpart, const float* __restrict__ Q,
                                     int ldq, const int* __restrict__ n_dev, int grid, int N,
                                     int D, float inv_var, double log_norm,
                                     double* __restrict__ logp, float* __restrict__ grad, int ldg) {
  const int n = *n_dev;
  const int row_tiles = (N + kNT - 1) / kNT;
  const int S = num_splits(n, grid, row_tiles);
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= n) return;
  const float* q = Q + (size_t)warp * ldq;
  double prior = 0.0;
  for (int d = lane; d < D; d += 32) {
    const float qd = q[d];
    float acc = 0.f;
    for (int s = 0; s < S; ++s) acc += gpart[((size_t)s * n + warp) * D + d];
    grad[(size_t)warp * ldg + d] = acc - qd * inv_var;
    prior += (double)qd * (double)qd;
  }
  prior = warp_sum(prior);
  if (lane == 0) {
    double lp = 0.0;
    for (int s = 0; s < S; ++s) lp += lpart[(size_t)s * n + warp];
    logp[warp] = lp - 0.5 * (double)inv_var * prior + (double)D * log_norm;
  }
}

class LogregSimt final : public Target {
 public:
  LogregSimt(gbm_context* ctx, const float* X, int64_t n, int64_t d, const float* y,
             float prior_scale)
      : N_(n), D_(d) {
    dim = d;
    ldx_ = (int)((d + 3) / 4 * 4);
    x_.reserve(sizeof(float) * (size_t)N_ * ldx_);
    y_.reserve(sizeof(float) * (size_t)N_);
    GBM_CUDA(cudaMemset2DAsync(x_.ptr, sizeof(float) * ldx_, 0, sizeof(float) * ldx_, N_,
                               ctx->stream));
    GBM_CUDA(cudaMemcpy2DAsync(x_.ptr, sizeof(float) * ldx_, X, sizeof(float) * d,
                               sizeof(float) * d, N_, cudaMemcpyDeviceToDevice, ctx->stream));
    GBM_CUDA(cudaMemcpyAsync(y_.ptr, y, sizeof(float) * N_, cudaMemcpyDeviceToDevice,
                             ctx->stream));
    inv_var_ = 1.f / (prior_scale * prior_scale);
    log_norm_ = -log((double)prior_scale) - 0.5 * log(2.0 * M_PI);
    grid_ = 2 * ctx->num_sms;
    kd_ = d <= 32 ? 2 : d <= 64 ? 4 : d <= 128 ? 8 : 16;
    smem_ = sizeof(float) * (size_t)(kd_ * 16) * (kCT + kXPad) + sizeof(float) * kNT * kCT;
    set_smem(kd_);
  }

  size_t workspace_bytes(int64_t cap) const override {
    const size_t rows = (size_t)grid_ * kCT + (size_t)cap;  // S * n <= grid * kCT + n
    return rows * sizeof(double) + rows * (size_t)D_ * sizeof(float) + 256;
  }

  // One launch covers at most grid_ * kCT chains (one work item per CTA);
  // larger batches run as consecutive chunks that share the workspace.
  void eval(const float* q, int ldq, const int* n_dev, int cap, double* logp, float* grad,
            int ldg, void* ws, cudaStream_t s) override {
    const size_t rows = (size_t)grid_ * kCT + (size_t)cap;
    double* lpart = static_cast<double*>(ws);
    float* gpart = reinterpret_cast<float*>(lpart + rows);
    const int N = (int)N_, D = (int)D_;
    const int lim = grid_ * kCT;
    for (int base = 0; base < cap; base += lim) {
      const float* qc = q + (size_t)base * ldq;
      const int g = work_grid(grid_, std::min(lim, cap - base), kCT, N_, kMinSplitRows);
      switch (kd_) {
        case 2: logreg_partial_kernel<2><<<g, kThreads, smem_, s>>>(
            x_.as<float>(), ldx_, y_.as<float>(), N, D, qc, ldq, n_dev, base, lim, g, lpart,
            gpart); break;
        case 4: logreg_partial_kernel<4><<<g, kThreads, smem_, s>>>(
            x_.as<float>(), ldx_, y_.as<float>(), N, D, qc, ldq, n_dev, base, lim, g, lpart,
            gpart); break;
        case 8: logreg_partial_kernel<8><<<g, kThreads, smem_, s>>>(
            x_.as<float>(), ldx_, y_.as<float>(), N, D, qc, ldq, n_dev, base, lim, g, lpart,
            gpart); break;
        default: logreg_partial_kernel<16><<<g, kThreads, smem_, s>>>(
            x_.as<float>(), ldx_, y_.as<float>(), N, D, qc, ldq, n_dev, base, lim, g, lpart,
            gpart); break;
      }
      GBM_CUDA(cudaGetLastError());
      launch_split_reduce(lpart, gpart, qc, ldq, n_dev, base, lim, std::min(lim, cap - base),
                          kCT, kNT, g, N, D, inv_var_, log_norm_, nullptr, logp + base,
                          grad + (size_t)base * ldg, ldg, s);
    }
  }

  int launches_per_eval(int64_t cap) const override {
    return 2 * (int)((cap + (int64_t)grid_ * kCT - 1) / ((int64_t)grid_ * kCT));
  }
  double flops(int64_t n) const override { return 4.0 * (double)N_ * D_ * n; }
  double bytes(int64_t n) const override {
    return 4.0 * (double)N_ * D_ + 4.0 * N_ + 8.0 * (double)n * D_ + 8.0 * n;
  }

 private:
  void set_smem(int kd) {
    const void* fn = kd == 2 ? (const void*)logreg_partial_kernel<2>
                   : kd == 4 ? (const void*)logreg_partial_kernel<4>
                   : kd == 8 ? (const void*)logreg_partial_kernel<8>
                             : (const void*)logreg_partial_kernel<16>;
    GBM_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_));
  }

  int64_t N_, D_;
  int ldx_ = 0, grid_ = 0, kd_ = 0;
  size_t smem_ = 0;
  float inv_var_ = 1.f;
  double log_norm_ = 0.0;
  DeviceBuffer x_, y_;
};

namespace {

} // namespace

std::unique_ptr<Target> make_logreg_simt(gbm_context* ctx, const float* X, int64_t n, int64_t d,
                                         const float* y, float prior_scale) {
  if (d > 256) return nullptr;
  if (d <= 128) return make_logreg_f32(ctx, X, n, d, y, prior_scale);
  return std::unique_ptr<Target>(new LogregSimt(ctx, X, n, d, y, prior_scale));
}

}  // namespace gbm

// ---------------------------------------------------------------------------
// Allocation-free logistic-regression log-density + gradient.
//
// Some callers cannot allocate device memory at all: code embedded in a host
// framework's custom-call or custom-op slot, which receives only the input
// and output buffers the framework owns and must not grow its own pool, and
// latency-bound serving loops that cannot afford the device-wide
// synchronisation cudaMalloc/cudaFree can cause.  For them this entry point
// keeps the kernel's scratch (the per-split partial log-likelihoods and
// gradients, and the batch-size word) in a fixed file-scope device array
// instead of a workspace.  The array occupies kNoAllocScratchBytes on every
// GPU that loads this library, for the life of the process.
// ---------------------------------------------------------------------------
#include <cstdio>
#include <mutex>
#include <string>
#include <vector>

#include "gb300_mcmc.h"

namespace {

constexpr size_t kNoAllocScratchBytes = 8u << 20;  // 8 MiB per device
constexpr size_t kNoAllocCountBytes = 256;          // batch-size word, padded

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

__global__ void noalloc_set_count(int* count, int n) { *count = n; }

struct NoAllocDevice {
  bool ready = false;
  unsigned char* scratch = nullptr;  // device address of g_noalloc_scratch
  int num_sms = 0;
};

std::mutex g_noalloc_mu;
std::vector<NoAllocDevice> g_noalloc_devices;

// Once per device, with that device current: resolve the device address of
// the scratch array (its host-side name is only a stand-in) and raise the
// kernels' dynamic shared-memory limit.  Allocates nothing on the device.
// The record is copied out while the lock is held: a first call on a
// higher-numbered device from another thread may grow the vector and move
// its elements.
int noalloc_setup(int device, NoAllocDevice* out) {
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if ((int)g_noalloc_devices.size() <= device) g_noalloc_devices.resize(device + 1);
  NoAllocDevice& d = g_noalloc_devices[device];
  if (!d.ready) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
      gbm::set_error(std::string("cudaGetSymbolAddress(g_noalloc_scratch): ") +
                     cudaGetErrorString(e));
      return GBM_ECUDA;
    }
    e = cudaDeviceGetAttribute(&d.num_sms, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) {
      gbm::set_error(std::string("cudaDeviceGetAttribute: ") + cudaGetErrorString(e));
      return GBM_ECUDA;
    }
    const int kds[4] = {2, 4, 8, 16};
    for (int kd : kds) {
      const size_t smem = sizeof(float) * (size_t)(kd * 16) * (gbm::kCT + gbm::kXPad) +
                          sizeof(float) * gbm::kNT * gbm::kCT;
      const void* fn = kd == 2 ? (const void*)gbm::logreg_partial_kernel<2>
                     : kd == 4 ? (const void*)gbm::logreg_partial_kernel<4>
                     : kd == 8 ? (const void*)gbm::logreg_partial_kernel<8>
                               : (const void*)gbm::logreg_partial_kernel<16>;
      e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) {
        gbm::set_error(std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e));
        return GBM_ECUDA;
      }
    }
    d.scratch = static_cast<unsigned char*>(p);
    d.ready = true;
  }
  *out = d;
  return GBM_OK;
}

}  // namespace

extern "C" int gbm_logreg_log_prob_and_grad_noalloc(const float* x, int64_t num_rows,
                                                    int64_t num_features, const float* y,
                                                    float prior_scale, const float* state,
                                                    int64_t chains, double* log_prob,
                                                    float* grad, void* cuda_stream) {
  if (!x || !y || !state || !log_prob || !grad) {
    gbm::set_error("gbm_logreg_log_prob_and_grad_noalloc: NULL argument");
    return GBM_EINVAL;
  }
  if (num_rows <= 0 || num_rows >= ((int64_t)1 << 31) || chains <= 0) {
    gbm::set_error("gbm_logreg_log_prob_and_grad_noalloc: need 0 < num_rows < 2^31, chains > 0");
    return GBM_EINVAL;
  }
  if (num_features <= 0 || num_features > 256) {
    gbm::set_error("gbm_logreg_log_prob_and_grad_noalloc: num_features must be in [1, 256]");
    return GBM_EINVAL;
  }
  if (!(prior_scale > 0.f)) {
    gbm::set_error("gbm_logreg_log_prob_and_grad_noalloc: prior_scale must be > 0");
    return GBM_EINVAL;
  }
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) {
    gbm::set_error(std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    return GBM_ECUDA;
  }
  NoAllocDevice dev;
  int st = noalloc_setup(device, &dev);
  if (st != GBM_OK) return st;

  // Scratch layout: [count word | lpart: rows doubles | gpart: rows * D floats],
  // rows = grid * kCT >= S * chains.  The grid shrinks as D grows so the
  // partials fit; chains is then limited to grid * kCT.
  const int D = (int)num_features, N = (int)num_rows;
  const size_t per_row = sizeof(double) + sizeof(float) * (size_t)D;
  const size_t avail = kNoAllocScratchBytes - kNoAllocCountBytes;
  int grid = 2 * dev.num_sms;
  const int fit = (int)(avail / (per_row * gbm::kCT));
  grid = std::min(grid, fit);
  if (grid < 1 || chains > (int64_t)grid * gbm::kCT) {
    char msg[256];
    snprintf(msg, sizeof(msg),
             "gbm_logreg_log_prob_and_grad_noalloc: %lld chains exceed the fixed %zu-byte "
             "scratch at %d features (maximum %d chains)",
             (long long)chains, kNoAllocScratchBytes, D, std::max(grid, 0) * gbm::kCT);
    gbm::set_error(msg);
    return GBM_EINVAL;
  }
  const int n = (int)chains;
  int* count = reinterpret_cast<int*>(dev.scratch);
  double* lpart = reinterpret_cast<double*>(dev.scratch + kNoAllocCountBytes);
  float* gpart = reinterpret_cast<float*>(lpart + (size_t)grid * gbm::kCT);
  cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
  const int kd = D <= 32 ? 2 : D <= 64 ? 4 : D <= 128 ? 8 : 16;
  const size_t smem = sizeof(float) * (size_t)(kd * 16) * (gbm::kCT + gbm::kXPad) +
                      sizeof(float) * gbm::kNT * gbm::kCT;
  const float inv_var = 1.f / (prior_scale * prior_scale);
  const double log_norm = -log((double)prior_scale) - 0.5 * log(2.0 * M_PI);
  noalloc_set_count<<<1, 1, 0, s>>>(count, n);
  switch (kd) {
    case 2: gbm::logreg_partial_kernel<2><<<grid, gbm::kThreads, smem, s>>>(
        x, D, y, N, D, state, D, count, 0, grid * gbm::kCT, grid, lpart, gpart); break;
    case 4: gbm::logreg_partial_kernel<4><<<grid, gbm::kThreads, smem, s>>>(
        x, D, y, N, D, state, D, count, 0, grid * gbm::kCT, grid, lpart, gpart); break;
    case 8: gbm::logreg_partial_kernel<8><<<grid, gbm::kThreads, smem, s>>>(
        x, D, y, N, D, state, D, count, 0, grid * gbm::kCT, grid, lpart, gpart); break;
    default: gbm::logreg_partial_kernel<16><<<grid, gbm::kThreads, smem, s>>>(
        x, D, y, N, D, state, D, count, 0, grid * gbm::kCT, grid, lpart, gpart); break;
  }
  gbm::logreg_reduce_kernel<<<(n + 7) / 8, 256, 0, s>>>(lpart, gpart, state, D, count, grid, N,
                                                         D, inv_var, log_norm, log_prob, grad, D);
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    gbm::set_error(std::string("gbm_logreg_log_prob_and_grad_noalloc launch: ") +
                   cudaGetErrorString(e));
    return GBM_ECUDA;
  }
  return GBM_OK;
}
