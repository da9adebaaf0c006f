// Fused logistic-regression log-density + gradient, FP32 CUDA cores, for up
// to 128 features (the plain FP32 form of the 1e5 x 100 workload).
//
// Mathematics (the inference_gym logistic-regression target,
// spinoffs/inference_gym/inference_gym/targets/logistic_regression.py:92-103,
// with the Bernoulli log-prob of distributions/bernoulli.py:126-140): for
// states q_c and z_rc = x_r . q_c,
//   log p(y_r | z) = y z - softplus(z) = (y - 1/2) z - |z|/2 - ln(1 + e^-|z|)
//   R_rc = y_r - sigmoid(z_rc) = (y_r - 1/2) - sign(z) (1/(1 + e^-|z|) - 1/2)
//   grad_c = X^T R_c - q_c / s^2.
// The linear part sum_r (y_r - 1/2) z_rc = (X^T (y - 1/2)) . q_c is added
// exactly (float64) by the split reduction; this kernel accumulates
// -(sum |z|/2 + sum ln(1 + e^-|z|)) and X^T R.
//
// Work decomposition: one CTA (256 threads, one per SM) owns a tile of 128
// chains and a contiguous range of 64-row tiles of X (a row split).  Per row
// tile, in FP32 on the CUDA cores:
//   phase 1  Z[64 rows][128 chains] = X_tile B^T: each thread 4 rows x 8
//            chains, K = features, 6 shared loads per 64 FMAs;
//   epilogue the log-likelihood sums and R (to shared memory);
//   phase 2  G[128 chains][Dp] += R^T X_tile: each thread 8 chains x KD
//            features (features f + 16 j), held in registers across the
//            CTA's rows, 4 + KD shared loads per 16 KD FMAs.
// X is stored on the device in row pairs, X2[N/2][Dp][2] (element (r, d) at
// ((r/2) Dp + d) 2 + r%2), zero-padded to Dp = 16 KD features and whole
// 64-row tiles, so that one 16-byte load gives phase 1 two rows x two
// features and one 8-byte load gives phase 2 two rows of one feature, and a
// row tile is one contiguous block moved by one bulk copy (cp.async.bulk)
// into a double-buffered shared-memory stage.  X is read from HBM once per
// chain tile (L2 serves the other chain tiles of the same rows).
#include <cuda_runtime.h>

#include <algorithm>
#include <memory>

#include "engine.h"
#include "split_reduce.cuh"
#include "tc_ptx.cuh"

namespace gbm {
namespace {

constexpr int kF32CT = 128;                 // chains per tile
constexpr int kF32RT = 64;                  // rows per tile
constexpr int kF32Threads = 256;
constexpr uint64_t kF32WaitNs = 2000000000ull;   // 2 s bound on every wait
constexpr int kF32TimeoutCode = 4;                // error word: bulk copy never landed
constexpr float kNegLog2e = -1.4426950408889634f;
constexpr float kLn2f = 0.6931471805599453f;

template <int KD>
struct F32Layout {
  static constexpr int kDp = 16 * KD;
  static constexpr int kBt = 0;                               // [Dp][128] float
  static constexpr int kXStage = kF32RT * kDp * 4;            // one row tile of X2
  static constexpr int kX = kBt + kDp * kF32CT * 4;           // 2 stages
  static constexpr int kY = kX + 2 * kXStage;                 // 2 x [64] float (y - 1/2)
  static constexpr int kR = kY + 2 * kF32RT * 4;              // [64][128] float
  static constexpr int kBar = kR + kF32RT * kF32CT * 4;       // 2 mbarriers + flag
  static constexpr int kBytes = kBar + 64;
  static_assert(16 * kF32CT * 8 <= kF32RT * kF32CT * 4, "reduction scratch fits R");
  static_assert(kBytes <= 232448, "shared memory over the sm_103a limit");
};

__host__ __device__ inline int f32_splits(int n, int grid, int row_tiles) {
  const int tiles = (n + kF32CT - 1) / kF32CT;
  if (tiles == 0) return 0;
  int s = grid / tiles;
  s = s < 1 ? 1 : s;
  return s > row_tiles ? row_tiles : s;
}

__device__ __forceinline__ float4 lds4(const float* p) {
  return *reinterpret_cast<const float4*>(p);
}

// -copysign(w, z): magnitude of w with the sign of -z.
__device__ __forceinline__ float neg_copysign_f(float w, float z) {
  return __int_as_float((__float_as_int(w) & 0x7fffffff) |
                        (~__float_as_int(z) & (int)0x80000000));
}

template <int KD>
__global__ void __launch_bounds__(kF32Threads, 1)
logreg_f32_kernel(const float* __restrict__ X2, const float* __restrict__ ym, int N, int D,
                  const float* __restrict__ Q, int ldq, const int* __restrict__ n_dev,
                  int c_base, int c_lim, int grid, double* __restrict__ lpart,
                  float* __restrict__ gpart, int* __restrict__ err) {
  using L = F32Layout<KD>;
  constexpr int Dp = L::kDp;
  extern __shared__ __align__(128) unsigned char smem[];
  const int n = chunk_count(*n_dev, c_base, c_lim);
  const int row_tiles = (N + kF32RT - 1) / kF32RT;
  const int S = f32_splits(n, grid, row_tiles);
  const int tiles = (n + kF32CT - 1) / kF32CT;
  if (S == 0 || (int)blockIdx.x >= tiles * S) return;
  const int tile = blockIdx.x % tiles, split = blockIdx.x / tiles;
  const int c0 = tile * kF32CT;
  const int rt_begin = (int)((long long)split * row_tiles / S);
  const int rt_end = (int)((long long)(split + 1) * row_tiles / S);
  const int T = rt_end - rt_begin;

  float* Bt = reinterpret_cast<float*>(smem + L::kBt);
  float* Xs = reinterpret_cast<float*>(smem + L::kX);
  float* Ys = reinterpret_cast<float*>(smem + L::kY);
  float* Rs = reinterpret_cast<float*>(smem + L::kR);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + L::kBar);
  const int tid = threadIdx.x;

  int issued = 0;              // thread 0: row tiles whose copies were issued
  auto issue = [&](int it) {   // thread 0: bulk copies of row tile rt_begin + it
    const int st = it & 1;
    issued = it + 1;
    const size_t r0 = (size_t)(rt_begin + it) * kF32RT;
    tc::fence_proxy_async_smem();
    tc::mbar_arrive_expect_tx(&full[st], (uint32_t)(L::kXStage + kF32RT * 4));
    tc::bulk_load(Xs + st * (L::kXStage / 4), X2 + r0 * Dp, (uint32_t)L::kXStage, &full[st]);
    tc::bulk_load(Ys + st * kF32RT, ym + r0, (uint32_t)(kF32RT * 4), &full[st]);
  };
  if (tid == 0) {
    tc::mbar_init(&full[0], 1);
    tc::mbar_init(&full[1], 1);
    tc::fence_mbar_init();
    if (T > 0) issue(0);
    if (T > 1) issue(1);
  }
  // Chain states, transposed: Bt[d][c] = Q[c0 + c][d], zero outside (n, D).
  for (int i = tid; i < Dp * kF32CT; i += kF32Threads) {
    const int c = i / Dp, d = i - c * Dp;
    Bt[d * kF32CT + c] = (c0 + c < n && d < D) ? Q[(size_t)(c0 + c) * ldq + d] : 0.f;
  }
  __syncthreads();

  const int ty = tid >> 4, tx = tid & 15;   // phase 1: rows 4 ty.., chains 4 tx.., 64 + 4 tx..
  const int cg = ty, fg = tx;               // phase 2: chains 4 cg.., 64 + 4 cg..; f = fg + 16 j
  const int dk = (D + 1) & ~1;              // K extent of phase 1 (B^T rows >= D are zero)
  float g[8][KD];
#pragma unroll
  for (int c = 0; c < 8; ++c)
#pragma unroll
    for (int j = 0; j < KD; ++j) g[c][j] = 0.f;
  // Per chain: Kahan sum over tiles of -(sum |z|/2 + sum ln(1 + e^-|z|)).
  float lsum[8], lcomp[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) lsum[c] = lcomp[c] = 0.f;
  bool ok = true;        // this thread's waits succeeded
  bool failed = false;   // some thread's wait ran out (uniform across the CTA)
  int it = 0;

  for (; it < T; ++it) {
    const int st = it & 1;
    if (!tc::mbar_wait(&full[st], (uint32_t)(it >> 1) & 1, kF32WaitNs)) ok = false;
    const float* xs = Xs + st * (L::kXStage / 4);
    // ---- phase 1: Z = X_tile B^T ----
    float z[4][8];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int c = 0; c < 8; ++c) z[i][c] = 0.f;
    const float* xa = xs + (2 * ty) * Dp * 2;        // row pair 2 ty (rows 4 ty, 4 ty + 1)
    const float* xb = xa + Dp * 2;                   // row pair 2 ty + 1
    const float* bp = Bt + 4 * tx;
    // Register double buffering: the next feature pair's six loads are in
    // flight while this pair's 64 FMAs issue (the last iteration re-reads
    // its own pair instead of reading past the tile).
    float4 u = lds4(xa), v = lds4(xb);   // x(r0,d) x(r1,d) x(r0,d+1) x(r1,d+1); rows r2, r3
    float4 b0 = lds4(bp), b1 = lds4(bp + 64), b2 = lds4(bp + kF32CT), b3 = lds4(bp + kF32CT + 64);
#pragma unroll 2
    for (int d = 0; d < dk; d += 2) {
      const int dn = d + 2 < dk ? d + 2 : d;
      const float4 un = lds4(xa + 2 * dn), vn = lds4(xb + 2 * dn);
      const float4 b0n = lds4(bp + dn * kF32CT), b1n = lds4(bp + dn * kF32CT + 64);
      const float4 b2n = lds4(bp + (dn + 1) * kF32CT), b3n = lds4(bp + (dn + 1) * kF32CT + 64);
      const float xr0[4] = {u.x, u.y, v.x, v.y};
      const float xr1[4] = {u.z, u.w, v.z, v.w};
      const float bb0[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
      const float bb1[8] = {b2.x, b2.y, b2.z, b2.w, b3.x, b3.y, b3.z, b3.w};
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int c = 0; c < 8; ++c) z[i][c] = fmaf(xr1[i], bb1[c], fmaf(xr0[i], bb0[c], z[i][c]));
      u = un; v = vn; b0 = b0n; b1 = b1n; b2 = b2n; b3 = b3n;
    }
    // ---- epilogue: log-likelihood sums and R ----
    const float4 yv = lds4(Ys + st * kF32RT + 4 * ty);
    const float yr[4] = {yv.x, yv.y, yv.z, yv.w};
    const int nvalid = N - (rt_begin + it) * kF32RT - 4 * ty;   // rows of mine that exist
    float sabs[8], prod[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) { sabs[c] = 0.f; prod[c] = 1.f; }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      float r[8];
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        const float a = fabsf(z[i][c]);
        const float e = tc::ex2_approx(a * kNegLog2e);       // e^-|z|
        const float u1 = 1.f + e;
        if (i < nvalid) {
          sabs[c] += a;
          prod[c] *= u1;
        }
        const float w = tc::rcp_approx(u1) - 0.5f;          // sigmoid(|z|) - 1/2
        r[c] = yr[i] + neg_copysign_f(w, z[i][c]);
      }
      float* rrow = Rs + (4 * ty + i) * kF32CT;
      *reinterpret_cast<float4*>(rrow + 4 * tx) = make_float4(r[0], r[1], r[2], r[3]);
      *reinterpret_cast<float4*>(rrow + 64 + 4 * tx) = make_float4(r[4], r[5], r[6], r[7]);
    }
#pragma unroll
    for (int c = 0; c < 8; ++c) {   // Kahan: lsum += -(sabs / 2 + ln prod)
      const float v = -fmaf(kLn2f, tc::lg2_approx(prod[c]), 0.5f * sabs[c]) - lcomp[c];
      const float t = lsum[c] + v;
      lcomp[c] = (t - lsum[c]) - v;
      lsum[c] = t;
    }
    if (__syncthreads_or(!ok)) {   // R complete (and every thread's wait succeeded)
      failed = true;
      break;
    }
    // ---- phase 2: G += R^T X_tile ----
    // Register double buffering of the residual rows and the row pair of X,
    // as in phase 1.
    const float* rp = Rs + 4 * cg;
    const float* xq = xs + 2 * fg;
    float4 ra0 = lds4(rp), ra1 = lds4(rp + 64), rb0 = lds4(rp + kF32CT),
           rb1 = lds4(rp + kF32CT + 64);
    float2 xv[KD];
#pragma unroll
    for (int j = 0; j < KD; ++j) xv[j] = *reinterpret_cast<const float2*>(xq + 32 * j);
#pragma unroll 2
    for (int p = 0; p < kF32RT / 2; ++p) {
      const int pn = p + 1 < kF32RT / 2 ? p + 1 : p;
      const float* rn = rp + (2 * pn) * kF32CT;
      const float4 ra0n = lds4(rn), ra1n = lds4(rn + 64), rb0n = lds4(rn + kF32CT),
                   rb1n = lds4(rn + kF32CT + 64);
      float2 xvn[KD];
#pragma unroll
      for (int j = 0; j < KD; ++j)
        xvn[j] = *reinterpret_cast<const float2*>(xq + pn * Dp * 2 + 32 * j);
      const float r0[8] = {ra0.x, ra0.y, ra0.z, ra0.w, ra1.x, ra1.y, ra1.z, ra1.w};
      const float r1[8] = {rb0.x, rb0.y, rb0.z, rb0.w, rb1.x, rb1.y, rb1.z, rb1.w};
#pragma unroll
      for (int j = 0; j < KD; ++j)
#pragma unroll
        for (int c = 0; c < 8; ++c)
          g[c][j] = fmaf(r1[c], xv[j].y, fmaf(r0[c], xv[j].x, g[c][j]));
      ra0 = ra0n; ra1 = ra1n; rb0 = rb0n; rb1 = rb1n;
#pragma unroll
      for (int j = 0; j < KD; ++j) xv[j] = xvn[j];
    }
    __syncthreads();   // stage st and R are free
    if (tid == 0 && it + 2 < T) issue(it + 2);
  }

  if (failed) {
    if (tid == 0) {
      tc::record_error(err, kF32TimeoutCode);
      // Let copies still in flight (tiles it .. issued - 1) land before the
      // CTA exits; each wait is bounded.
      for (int j = it; j < issued; ++j)
        tc::mbar_wait(&full[j & 1], (uint32_t)(j >> 1) & 1, kF32WaitNs);
    }
    return;
  }
  // Per-chain log-likelihood partial: sum the 16 row groups in fixed order.
  double* red = reinterpret_cast<double*>(Rs);     // [16][128]
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const int cc = c < 4 ? 4 * tx + c : 64 + 4 * tx + (c - 4);
    red[ty * kF32CT + cc] = (double)lsum[c] - (double)lcomp[c];
  }
  __syncthreads();
  if (tid < kF32CT && c0 + tid < n) {
    double s = 0.0;
#pragma unroll
    for (int t = 0; t < 16; ++t) s += red[t * kF32CT + tid];
    lpart[(size_t)split * n + c0 + tid] = s;
  }
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    const int cc = c0 + (c < 4 ? 4 * cg + c : 64 + 4 * cg + (c - 4));
    if (cc >= n) continue;
    float* dst = gpart + ((size_t)split * n + cc) * D;
#pragma unroll
    for (int j = 0; j < KD; ++j) {
      const int d = fg + 16 * j;
      if (d < D) dst[d] = g[c][j];
    }
  }
}

// X [N][D] -> X2 [N2/2][Dp][2] (row pairs, zero padding) and ym = y - 1/2
// (zero past N), N2 = N rounded up to whole row tiles.
__global__ void f32_pack_kernel(const float* __restrict__ X, const float* __restrict__ y,
                                int64_t N, int D, int Dp, int64_t N2, float* __restrict__ X2,
                                float* __restrict__ ym) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N2) ym[i] = i < N ? y[i] - 0.5f : 0.f;
  if (i >= N2 * Dp) return;
  const int64_t r = i / Dp;
  const int d = (int)(i - r * Dp);
  X2[((r >> 1) * Dp + d) * 2 + (r & 1)] = (r < N && d < D) ? X[r * D + d] : 0.f;
}

// lin[d] = sum_r (y_r - 1/2) X[r][d] in float64 and a fixed order: block b
// sums rows [b chunk, (b + 1) chunk) into part[b][d]; blocks added in order.
__global__ void f32_lin_partial(const float* __restrict__ X, const float* __restrict__ y,
                                int64_t N, int D, int64_t chunk, double* __restrict__ part) {
  const int64_t r0 = (int64_t)blockIdx.x * chunk;
  const int64_t r1 = r0 + chunk < N ? r0 + chunk : N;
  for (int d = threadIdx.x; d < D; d += blockDim.x) {
    double acc = 0.0;
    for (int64_t r = r0; r < r1; ++r) acc += ((double)y[r] - 0.5) * (double)X[r * D + d];
    part[(size_t)blockIdx.x * D + d] = acc;
  }
}

__global__ void f32_lin_sum(const double* __restrict__ part, int nb, int D,
                            double* __restrict__ lin) {
  const int d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= D) return;
  double acc = 0.0;
  for (int b = 0; b < nb; ++b) acc += part[(size_t)b * D + d];
  lin[d] = acc;
}

template <int KD>
void f32_set_smem() {
  GBM_CUDA(cudaFuncSetAttribute(logreg_f32_kernel<KD>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                F32Layout<KD>::kBytes));
}

class LogregF32 final : public Target {
 public:
  LogregF32(gbm_context* ctx, const float* X, int64_t n, int64_t d, const float* y,
            float prior_scale)
      : N_(n), D_(d) {
    dim = d;
    kd_ = (int)((d + 15) / 16);
    if (kd_ == 5) kd_ = 6;   // instantiated widths: 1 2 3 4 6 7 8
    dp_ = 16 * kd_;
    n2_ = (n + kF32RT - 1) / kF32RT * kF32RT;
    x2_.reserve(sizeof(float) * (size_t)n2_ * dp_);
    ym_.reserve(sizeof(float) * (size_t)n2_);
    const int64_t total = n2_ * dp_;
    f32_pack_kernel<<<(unsigned)((total + 255) / 256), 256, 0, ctx->stream>>>(
        X, y, N_, (int)D_, dp_, n2_, x2_.as<float>(), ym_.as<float>());
    GBM_CUDA(cudaGetLastError());
    {
      const int nb = 2 * ctx->num_sms;
      const int64_t chunk = (N_ + nb - 1) / nb;
      DeviceBuffer part;
      part.reserve(sizeof(double) * (size_t)nb * D_);
      lin_.reserve(sizeof(double) * (size_t)D_);
      f32_lin_partial<<<nb, 128, 0, ctx->stream>>>(X, y, N_, (int)D_, chunk,
                                                   part.as<double>());
      f32_lin_sum<<<(unsigned)((D_ + 127) / 128), 128, 0, ctx->stream>>>(
          part.as<double>(), nb, (int)D_, lin_.as<double>());
      GBM_CUDA(cudaGetLastError());
      GBM_CUDA(cudaStreamSynchronize(ctx->stream));   // `part` is freed on scope exit
    }
    inv_var_ = 1.f / (prior_scale * prior_scale);
    log_norm_ = -log((double)prior_scale) - 0.5 * log(2.0 * M_PI);
    grid_ = ctx->num_sms;
    err_dev_ = ctx->err_dev;
    switch (kd_) {
      case 1: f32_set_smem<1>(); break;
      case 2: f32_set_smem<2>(); break;
      case 3: f32_set_smem<3>(); break;
      case 4: f32_set_smem<4>(); break;
      case 6: f32_set_smem<6>(); break;
      case 7: f32_set_smem<7>(); break;
      default: f32_set_smem<8>(); break;
    }
  }

  size_t workspace_bytes(int64_t cap) const override {
    const size_t rows = (size_t)grid_ * kF32CT + (size_t)cap;
    return rows * sizeof(double) + rows * (size_t)D_ * sizeof(float) + 256;
  }

  // One launch covers at most grid_ * 128 chains (one work item per CTA);
  // larger batches run as consecutive chunks that share the workspace.
  void eval(const float* q, int ldq, const int* n_dev, int cap, double* logp, float* grad,
            int ldg, void* ws, cudaStream_t s) override {
    const size_t rows = (size_t)grid_ * kF32CT + (size_t)cap;
    double* lpart = static_cast<double*>(ws);
    float* gpart = reinterpret_cast<float*>(lpart + rows);
    const int N = (int)N_, D = (int)D_;
    const int lim = grid_ * kF32CT;
    for (int base = 0; base < cap; base += lim) {
      const float* qc = q + (size_t)base * ldq;
      const int g = work_grid(grid_, std::min(lim, cap - base), kF32CT, N_, kMinSplitRows);
#define GBM_F32_LAUNCH(KD_)                                                                \
  logreg_f32_kernel<KD_><<<g, kF32Threads, F32Layout<KD_>::kBytes, s>>>(                    \
      x2_.as<float>(), ym_.as<float>(), N, D, qc, ldq, n_dev, base, lim, g, lpart, gpart,     \
      err_dev_)
      switch (kd_) {
        case 1: GBM_F32_LAUNCH(1); break;
        case 2: GBM_F32_LAUNCH(2); break;
        case 3: GBM_F32_LAUNCH(3); break;
        case 4: GBM_F32_LAUNCH(4); break;
        case 6: GBM_F32_LAUNCH(6); break;
        case 7: GBM_F32_LAUNCH(7); break;
        default: GBM_F32_LAUNCH(8); break;
      }
#undef GBM_F32_LAUNCH
      GBM_CUDA(cudaGetLastError());
      launch_split_reduce(lpart, gpart, qc, ldq, n_dev, base, lim, std::min(lim, cap - base),
                          kF32CT, kF32RT, g, N, D, inv_var_, log_norm_, lin_.as<double>(),
                          logp + base, grad + (size_t)base * ldg, ldg, s);
    }
  }

  int launches_per_eval(int64_t cap) const override {
    return 2 * (int)((cap + (int64_t)grid_ * kF32CT - 1) / ((int64_t)grid_ * kF32CT));
  }
  double flops(int64_t n) const override { return 4.0 * (double)N_ * D_ * n; }
  double bytes(int64_t n) const override {
    return 4.0 * (double)N_ * D_ + 4.0 * N_ + 8.0 * (double)n * D_ + 8.0 * n;
  }

 private:
  int64_t N_, D_, n2_ = 0;
  int kd_ = 1, dp_ = 16, grid_ = 0;
  float inv_var_ = 1.f;
  double log_norm_ = 0.0;
  int* err_dev_ = nullptr;
  DeviceBuffer x2_, ym_, lin_;
};

}  // namespace

std::unique_ptr<Target> make_logreg_f32(gbm_context* ctx, const float* X, int64_t n, int64_t d,
                                        const float* y, float prior_scale) {
  if (d > 128) return nullptr;
  return std::unique_ptr<Target>(new LogregF32(ctx, X, n, d, y, prior_scale));
}

}  // namespace gbm
