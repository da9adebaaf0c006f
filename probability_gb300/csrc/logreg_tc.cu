// Mixed-precision fused logistic-regression log-density + gradient on the
// 5th-generation tensor cores (tcgen05, TMEM accumulators, TMA).
//
// Same mathematics as logreg_simt.cu (the inference_gym logistic-regression
// target, spinoffs/inference_gym/inference_gym/targets/logistic_regression.py:
// 92-103; distributions/bernoulli.py:126-140): per 128-row tile of X and
// tile of chains,
//   Z = X_tile B^T,  R = y - sigmoid(Z),  logp += sum_rows log Bernoulli(y | Z),
//   G += X_tile^T R,
// with BF16 operands and FP32 accumulation in TMEM.  X is BF16 (plus a BF16
// residual X_lo for FP32 data up to 128 features); the FP32 chain states B
// are split into a BF16 high part and a BF16 residual and both are
// multiplied (residual correction), so Z -- and therefore the log-density
// that drives acceptance -- carries ~16 significant bits of the states.  In
// the chain-major kernel (D <= 128) the gradient contraction is corrected
// the same way: R is split into BF16 hi + lo and G = R_hi^T X_hi +
// R_lo^T X_hi (+ R_hi^T X_lo for FP32 data); above 128 features R enters
// the gradient contraction as BF16.  A gradient that is a
// deterministic function of the state keeps the leapfrog map reversible and
// volume-preserving, so the sampler stays exact; only its acceptance rate
// depends on the gradient's accuracy.
//
// Three kernels, by feature count:
//   D <= 128        logreg_tct_kernel: chain-major (states and R in TMEM as
//                   the A operand; one thread per chain in the epilogue);
//   128 < D <= 256  logreg_tc_kernel: row-major (X tile as the A operand of
//                   both contractions, R through shared memory);
//   256 < D <= 512  logreg_tc_pair_kernel: a 2-CTA cluster splits the
//                   features of the row-major form.
// In all three one X tile in shared memory (TMA, 128-byte swizzle,
// [64-feature block][128 rows][128 B]) serves both contractions, read K-major
// by the first and MN-major by the second, so X is read from HBM/L2 once per
// chain tile.  Warp 0 issues TMA loads, warp 1 allocates TMEM and issues the
// MMAs, the other warps run the epilogue.  Every wait is bounded
// (%globaltimer); on timeout a kernel records an error code, drains what it
// issued and frees its TMEM.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <memory>
#include <cstdlib>
#include <string>

#include "engine.h"
#include "split_reduce.cuh"
#include "tc_ptx.cuh"

namespace gbm {
namespace {

constexpr int kRows = 128;                         // rows of X per tile
// Threads of a CTA with EPI epilogue warps (plus the TMA and MMA warps).
__host__ __device__ constexpr int tc_threads(int epi) { return 32 * (2 + epi); }
constexpr uint64_t kWaitLimitNs = 2000000000ull;   // 2 s bound on every device wait
constexpr float kNeg2Log2e = -2.8853900817779268f;  // -2 log2(e)
constexpr float kLn2 = 0.6931471805599453f;

enum TcError : int {
  kTcOk = 0,
  kTcTimeoutTma = 1,
  kTcTimeoutMma = 2,
  kTcTimeoutEpilogue = 3,
};

__host__ __device__ inline int tc_splits(int n, int ct, int grid, int row_tiles) {
  const int tiles = (n + ct - 1) / ct;
  if (tiles == 0) return 0;
  int s = grid / tiles;
  s = s < 1 ? 1 : s;
  return s > row_tiles ? row_tiles : s;
}

// Shared memory of the row-major kernel (instantiated for 128 < D <= 256:
// KB = 4, 64-chain tiles).  KB = 2 would give X_hi three stages, so that the
// TMA refill of a stage (which can start only once GEMM2 has read it) runs a
// full tile ahead of the GEMM1 that needs it, and a single R buffer.
template <int KB, int CT, bool XLO>
struct TcLayout {
  static constexpr int kStages = KB == 2 ? 3 : 2;      // X_hi stages
  static constexpr int kRBufs = KB == 2 ? 1 : 2;       // R buffers
  static constexpr int kXStage = KB * 16384;           // [KB][128 rows][128 B]
  static constexpr int kBBytes = KB * CT * 128;        // [KB][CT rows][128 B]
  static constexpr int kRBuf = (CT / 64) * 16384;      // [CT/64][128 rows][128 B]
  static constexpr int kX = 0;
  static constexpr int kBhi = kX + kStages * kXStage;
  static constexpr int kBlo = kBhi + kBBytes;
  static constexpr int kR = kBlo + kBBytes;
  static constexpr int kXlo = kR + kRBufs * kRBuf;     // X residual, 1 stage (XLO only)
  static constexpr int kCtl = kXlo + (XLO ? kXStage : 0);  // barriers + tmem slot + abort
  // After the last MMA the R buffers are reused for the [4 quarters][CT]
  // double log-likelihood reduction.
  static constexpr int kRed = kR;
  static constexpr int kBytes = kCtl + 256;
  static_assert(4 * CT * 8 <= kRBufs * kRBuf, "reduction scratch must fit the R buffers");
  static constexpr int kMTiles = KB / 2;               // 128-feature tiles of G
  static constexpr uint32_t kTmemCols = (2 * CT + kMTiles * CT) <= 256 ? 256 : 512;
  static_assert(kBytes + 1024 <= 232448, "shared memory over the sm_103a limit");
};

struct Bars {
  uint64_t x_full[3], x_empty[3], z_full[2], z_empty[2], r_full[2], r_empty[2], g_done, drain;
  uint64_t xlo_full, xlo_empty;
};

__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
  __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t*>(&v);
}

// R = y - sigmoid(z) for two elements, from h = z / 2: sigmoid(z) = 1/2 +
// tanh(h) / 2, so R = (y - 1/2) - tanh(h) / 2, rounded to nearest BF16 (the
// contraction's operand type; round-to-nearest keeps the rounding unbiased,
// which matters for the intercept column, whose gradient sums R over all
// rows).
__device__ __forceinline__ uint32_t residual_bf16x2(float h0, float h1, float ym) {
  return pack_bf16x2(fmaf(-0.5f, tc::tanh_approx(h0), ym), fmaf(-0.5f, tc::tanh_approx(h1), ym));
}

__device__ __forceinline__ void named_barrier(int id, int nthreads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// Wait that also gives up when another role has already aborted.
__device__ __forceinline__ bool wait_or_abort(uint64_t* bar, uint32_t parity,
                                              volatile int* abort_flag) {
  if (tc::mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = tc::globaltimer_ns();
  while (true) {
    if (tc::mbar_try_wait(bar, parity)) return true;
    if (*abort_flag) return false;
    if (tc::globaltimer_ns() - t0 > kWaitLimitNs) return false;
  }
}

// wait_or_abort by every lane of a warp, with one outcome for the whole warp
// (the .sync.aligned TMEM accesses that follow need a converged warp).
__device__ __forceinline__ bool warp_wait(uint64_t* bar, uint32_t parity,
                                          volatile int* abort_flag) {
  return __all_sync(0xffffffffu, wait_or_abort(bar, parity, abort_flag));
}

// XLO: X is FP32 data stored as X_hi + X_lo (both BF16); GEMM1 adds the
// X_lo B_hi product so Z keeps ~16 significant bits of the FP32 data.  The
// gradient contraction uses X_hi.
template <int KB, int CT, int EPI, bool XLO>
__global__ void __launch_bounds__(tc_threads(EPI), 1)
logreg_tc_kernel(const __grid_constant__ CUtensorMap xmap,
                 const __grid_constant__ CUtensorMap xlomap, const float* __restrict__ y, int N,
                 int D, const float* __restrict__ Q, int ldq, const int* __restrict__ n_dev,
                 int c_base, int c_lim, int grid, double* __restrict__ lpart,
                 float* __restrict__ gpart, int* __restrict__ err) {
  using L = TcLayout<KB, CT, XLO>;
  constexpr int kThreads = tc_threads(EPI);
  constexpr int kCW = CT * 4 / EPI;             // chains per epilogue warp
  static_assert(kCW == 32 || kCW == 64, "epilogue width");
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int n = chunk_count(*n_dev, c_base, c_lim);
  const int row_tiles = (N + kRows - 1) / kRows;
  const int S = tc_splits(n, CT, grid, row_tiles);
  const int tiles = (n + CT - 1) / CT;
  if (S == 0 || (int)blockIdx.x >= tiles * S) return;
  const int tile = blockIdx.x % tiles, split = blockIdx.x / tiles;
  const int c0 = tile * CT;
  const int rt_begin = (int)((long long)split * row_tiles / S);
  const int rt_end = (int)((long long)(split + 1) * row_tiles / S);
  const int T = rt_end - rt_begin;

  unsigned char* Xs = smem + L::kX;
  unsigned char* Bhi = smem + L::kBhi;
  unsigned char* Blo = smem + L::kBlo;
  unsigned char* Rs = smem + L::kR;
  Bars* bars = reinterpret_cast<Bars*>(smem + L::kCtl);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + L::kCtl + sizeof(Bars));
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
  double* red = reinterpret_cast<double*>(smem + L::kRed);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    for (int i = 0; i < 3; ++i) {
      tc::mbar_init(&bars->x_full[i], 1);
      tc::mbar_init(&bars->x_empty[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      tc::mbar_init(&bars->z_full[i], 1);
      tc::mbar_init(&bars->z_empty[i], EPI);
      tc::mbar_init(&bars->r_full[i], EPI);
      tc::mbar_init(&bars->r_empty[i], 1);
    }
    tc::mbar_init(&bars->g_done, 1);
    tc::mbar_init(&bars->drain, 1);
    tc::mbar_init(&bars->xlo_full, 1);
    tc::mbar_init(&bars->xlo_empty, 1);
    *abort_flag = 0;
    tc::fence_mbar_init();
    tc::prefetch_tmap(&xmap);
  }
  if (warp == 1) tc::tmem_alloc(tmem_slot, L::kTmemCols);

  // Chain states / 2 -> BF16 hi/lo, K-major 128-byte-swizzled [KB][CT][128 B].
  // The factor 1/2 (exact) makes the accumulator hold h = z / 2, the argument
  // the epilogue needs for both tanh and exp.
  for (int i = tid; i < CT * KB * 8; i += kThreads) {
    const int c = i / (KB * 8), chunk = i % (KB * 8);
    const int d0 = chunk * 8;
    float v[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const int d = d0 + e;
      v[e] = (c0 + c < n && d < D) ? 0.5f * Q[(size_t)(c0 + c) * ldq + d] : 0.f;
    }
    uint32_t hi[4], lo[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const __nv_bfloat162 h = __floats2bfloat162_rn(v[2 * e], v[2 * e + 1]);
      hi[e] = *reinterpret_cast<const uint32_t*>(&h);
      const float2 hf = __bfloat1622float2(h);
      lo[e] = pack_bf16x2(v[2 * e] - hf.x, v[2 * e + 1] - hf.y);
    }
    const uint32_t off = (d0 >> 6) * (CT * 128) + tc::sw128_offset(c, d0 & 63);
    *reinterpret_cast<uint4*>(Bhi + off) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
    *reinterpret_cast<uint4*>(Blo + off) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
  }
  tc::fence_proxy_async_smem();
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      int it = 0;
      for (; it < T; ++it) {
        const int s = it % L::kStages;
        const uint32_t use = (uint32_t)(it / L::kStages);
        if (!wait_or_abort(&bars->x_empty[s], (use & 1) ^ 1, abort_flag)) {
          tc::record_error(err,kTcTimeoutTma);
          *abort_flag = 1;
          break;
        }
        tc::mbar_arrive_expect_tx(&bars->x_full[s], L::kXStage);
#pragma unroll
        for (int kb = 0; kb < KB; ++kb)
          tc::tma_load_2d(Xs + s * L::kXStage + kb * 16384, &xmap, kb * 64,
                          (rt_begin + it) * kRows, &bars->x_full[s]);
        if constexpr (XLO) {
          // Single X_lo buffer: free once GEMM1 of the previous tile is done.
          if (!wait_or_abort(&bars->xlo_empty, (uint32_t)(it & 1) ^ 1, abort_flag)) {
            tc::record_error(err, kTcTimeoutTma);
            *abort_flag = 1;
            ++it;
            break;
          }
          tc::mbar_arrive_expect_tx(&bars->xlo_full, L::kXStage);
#pragma unroll
          for (int kb = 0; kb < KB; ++kb)
            tc::tma_load_2d(smem + L::kXlo + kb * 16384, &xlomap, kb * 64,
                            (rt_begin + it) * kRows, &bars->xlo_full);
        }
      }
      // Drain: every issued load has landed before the CTA can exit.
      for (int j = (it > L::kStages ? it - L::kStages : 0); j < it; ++j)
        tc::mbar_wait(&bars->x_full[j % L::kStages], (uint32_t)((j / L::kStages) & 1),
                      kWaitLimitNs);
      if constexpr (XLO) {
        if (it > 0) tc::mbar_wait(&bars->xlo_full, (uint32_t)((it - 1) & 1), kWaitLimitNs);
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      constexpr uint32_t idesc1 = tc::idesc_bf16_f32(128, CT, false, false);  // K-major A, B
      constexpr uint32_t idesc2 = tc::idesc_bf16_f32(128, CT, true, true);    // MN-major A, B
      const uint32_t xs_a = tc::smem_u32(Xs), bhi_a = tc::smem_u32(Bhi);
      const uint32_t blo_a = tc::smem_u32(Blo), rs_a = tc::smem_u32(Rs);
      const uint32_t tg = tmem + 2 * CT;
      const int ksteps = (D + 15) >> 4;   // K-steps of 16 features holding data
      bool ok = true;
      auto gemm1 = [&](int it) -> bool {
        const int s = it % L::kStages, b = it & 1;
        if (!wait_or_abort(&bars->x_full[s], (uint32_t)(it / L::kStages) & 1, abort_flag))
          return false;
        if (!wait_or_abort(&bars->z_empty[b], ((uint32_t)(it >> 1) & 1) ^ 1, abort_flag))
          return false;
        if constexpr (XLO) {
          if (!wait_or_abort(&bars->xlo_full, (uint32_t)(it & 1), abort_flag)) return false;
        }
        tc::tc_fence_after();
        const uint32_t tz = tmem + b * CT;
        const uint32_t xa = xs_a + s * L::kXStage;
        const uint32_t xla = tc::smem_u32(smem + L::kXlo);
#pragma unroll
        for (int kb = 0; kb < KB; ++kb) {
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            if (kb * 4 + k >= ksteps) break;   // all-zero padding features
            const uint64_t a = tc::smem_desc_sw128(xa + kb * 16384 + k * 32, 16, 1024);
            const uint64_t bh = tc::smem_desc_sw128(bhi_a + kb * (CT * 128) + k * 32, 16, 1024);
            const uint64_t bl = tc::smem_desc_sw128(blo_a + kb * (CT * 128) + k * 32, 16, 1024);
            tc::mma_bf16(tz, a, bh, idesc1, (kb | k) ? 1u : 0u);
            tc::mma_bf16(tz, a, bl, idesc1, 1u);
            if constexpr (XLO) {
              const uint64_t al = tc::smem_desc_sw128(xla + kb * 16384 + k * 32, 16, 1024);
              tc::mma_bf16(tz, al, bh, idesc1, 1u);
            }
          }
        }
        tc::mma_commit(&bars->z_full[b]);
        if constexpr (XLO) tc::mma_commit(&bars->xlo_empty);
        return true;
      };
      if (T > 0) ok = gemm1(0);
      for (int it = 0; it < T && ok; ++it) {
        if (it + 1 < T) {
          ok = gemm1(it + 1);
          if (!ok) break;
        }
        const int s = it % L::kStages, rb = it % L::kRBufs;
        if (!wait_or_abort(&bars->r_full[rb], (uint32_t)(it / L::kRBufs) & 1, abort_flag)) {
          ok = false;
          break;
        }
        tc::tc_fence_after();
        const uint32_t xa = xs_a + s * L::kXStage;
        const uint32_t ra = rs_a + rb * L::kRBuf;
#pragma unroll
        for (int mt = 0; mt < L::kMTiles; ++mt) {
#pragma unroll
          for (int ks = 0; ks < kRows / 16; ++ks) {
            const uint64_t a = tc::smem_desc_sw128(xa + mt * 32768 + ks * 2048, 16384, 1024);
            const uint64_t bd = tc::smem_desc_sw128(ra + ks * 2048, 16384, 1024);
            tc::mma_bf16(tg + mt * CT, a, bd, idesc2, (it > 0 || ks > 0) ? 1u : 0u);
          }
        }
        tc::mma_commit(&bars->x_empty[s]);
        tc::mma_commit(&bars->r_empty[rb]);
      }
      if (ok) {
        tc::mma_commit(&bars->g_done);
      } else {
        tc::record_error(err,kTcTimeoutMma);
        *abort_flag = 1;
      }
      // Drain: all MMAs issued by this thread have completed.
      tc::mma_commit(&bars->drain);
      tc::mbar_wait(&bars->drain, 0, kWaitLimitNs);
    }
  } else {
    // ---------------- epilogue (EPI warps) ----------------
    const int quarter = warp & 3;                 // TMEM lanes 32*quarter ..
    const int half = (warp - 2) >> 2;             // chains [half*kCW, +kCW)
    const uint32_t lane_base = (uint32_t)(quarter * 32) << 16;
    const int r = quarter * 32 + lane;            // row of the tile this thread owns
    // Per chain: softplus(z) = max(z, 0) + ln(1 + e^-|z|) and max(z, 0) =
    // z/2 + |h|, so sum_r log Bernoulli(y_r | z_r) = sum_r (y_r - 1/2) z_r
    // - sum_r (|h_r| + ln(1 + e^-|z_r|)).  The first sum is linear in the
    // state and is added exactly by the reduction; sacc accumulates the
    // second (one accumulator per chain leaves room for the whole row of Z
    // in registers: one TMEM load and one wait per tile).
    float sacc[kCW];
#pragma unroll
    for (int c = 0; c < kCW; ++c) sacc[c] = 0.f;
    bool ok = true;
    // y of this thread's row, prefetched one tile ahead.
    float y_next = 0.f;
    {
      const int row0 = rt_begin * kRows + r;
      if (T > 0 && row0 < N) y_next = y[row0];
    }
    for (int it = 0; it < T; ++it) {
      const int b = it & 1, rb = it % L::kRBufs;
      if (!wait_or_abort(&bars->z_full[b], (uint32_t)(it >> 1) & 1, abort_flag)) {
        ok = false;
        break;
      }
      tc::tc_fence_after();
      const int row = (rt_begin + it) * kRows + r;
      const bool valid = row < N;
      const float ym = (valid ? y_next : 0.f) - 0.5f;
      if (it + 1 < T && row + kRows < N) y_next = y[row + kRows];
      const uint32_t tz = tmem + b * CT + half * kCW;
      unsigned char* Rb = Rs + rb * L::kRBuf;
      float h[kCW];
#pragma unroll
      for (int q = 0; q < kCW / 32; ++q) tc::tmem_ld32(tz + lane_base + q * 32, h + q * 32);
      tc::tmem_ld_wait();
      bool r_free = false;
#pragma unroll
      for (int g8 = 0; g8 < kCW / 8; ++g8) {
        uint32_t rp[4] = {0u, 0u, 0u, 0u};                   // rows past N: R = 0
        if (valid) {
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const float a = fabsf(h[g8 * 8 + j]);
            const float t = tc::ex2_approx(a * kNeg2Log2e);     // e^-|z|
            sacc[g8 * 8 + j] += fmaf(kLn2, tc::lg2_approx(1.f + t), a);
          }
#pragma unroll
          for (int j = 0; j < 4; ++j)
            rp[j] = residual_bf16x2(h[g8 * 8 + 2 * j], h[g8 * 8 + 2 * j + 1], ym);
        }
        if (g8 == 0) {
          // GEMM2 of the tile that last used this R buffer must be done.
          r_free = wait_or_abort(&bars->r_empty[rb], ((uint32_t)(it / L::kRBufs) & 1) ^ 1,
                                 abort_flag);
          if (!r_free) break;
        }
        const int c = half * kCW + g8 * 8;
        *reinterpret_cast<uint4*>(Rb + (c >> 6) * 16384 + tc::sw128_offset(r, c & 63)) =
            make_uint4(rp[0], rp[1], rp[2], rp[3]);
      }
      if (!r_free) {
        ok = false;
        break;
      }
      tc::tc_fence_before();
      tc::fence_proxy_async_smem();
      __syncwarp();
      if (lane == 0) {
        tc::mbar_arrive(&bars->z_empty[b]);
        tc::mbar_arrive(&bars->r_full[rb]);
      }
    }
    if (ok && T > 0) ok = wait_or_abort(&bars->g_done, 0, abort_flag);
    if (!ok) {
      tc::record_error(err,kTcTimeoutEpilogue);
      *abort_flag = 1;
    } else {
      tc::tc_fence_after();
      // Gradient partials: TMEM lane = feature, column = chain.
#pragma unroll
      for (int mt = 0; mt < L::kMTiles; ++mt) {
        const int d = mt * 128 + quarter * 32 + lane;
#pragma unroll
        for (int ch = 0; ch < kCW / 16; ++ch) {
          float g[16];
          tc::tmem_ld16(tmem + 2 * CT + mt * CT + half * kCW + lane_base + ch * 16, g);
          tc::tmem_ld_wait();
          if (d < D) {
#pragma unroll
            for (int j = 0; j < 16; ++j) {
              const int c = c0 + half * kCW + ch * 16 + j;
              if (c < n) gpart[((size_t)split * n + c) * D + d] = g[j];
            }
          }
        }
      }
      // Nonlinear log-likelihood partials: minus the sum over the 128 rows per
      // chain (FP32 shuffles: the FP64 pipe of this GPU is far too narrow for
      // a per-chain warp reduction; only the final 4-way sum is FP64).
#pragma unroll
      for (int c = 0; c < kCW; ++c) {
        float v = -sacc[c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[quarter * CT + half * kCW + c] = (double)v;
      }
    }
    named_barrier(1, 32 * EPI);
    if (ok) {
      for (int c = tid - 64; c < CT; c += 32 * EPI) {
        const double sum = red[c] + red[CT + c] + red[2 * CT + c] + red[3 * CT + c];
        if (c0 + c < n) lpart[(size_t)split * n + c0 + c] = sum;
      }
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem, L::kTmemCols);
  }
}

// ---------------------------------------------------------------------------
// D <= 128, chain-major: the chain states stay in TMEM as the A operand of
// both contractions, so every MMA reads only X from shared memory (half the
// shared-memory traffic of the row-major form above):
//   Z^T  = B X_tile^T        (M = 128 chains, N = 128 rows, K = features)
//   R^T  = (y - sigmoid(Z))^T, BF16, written back to TMEM by the epilogue
//   G^T += R^T X_tile        (M = 128 chains, N = features, K = 128 rows)
// B is stored in TMEM as BF16 hi/lo (residual correction, as above); X_tile
// is the same swizzled shared-memory tile, read K-major by the first MMA and
// MN-major by the second.
//
// Each epilogue thread owns one chain (its TMEM lane) and 32 rows of a tile,
// which changes the arithmetic per element:
//   * sum_r ln(1 + e^-|z_r|) = ln prod_r (1 + e^-|z_r|): one lg2 per 32 rows
//     (each factor is in (1, 2], so a product of 16 stays below 2^16);
//   * sigmoid(|z|) = 1 / (1 + e^-|z|) by the hardware reciprocal;
//   * the FP32 arithmetic around them runs two rows per instruction (packed
//     f32x2), since instruction issue, not the multi-function unit, is the
//     scarce resource of this epilogue.
//
// TMEM columns: B_hi [0, 64), B_lo [64, 128), two Z^T buffers [128, 256) and
// [256, 384), G^T [384, 512).  R^T overwrites, in place, the first 16 of the
// 32 Z^T columns the same warp has just loaded; each 16-row K-step of the
// second contraction reads 8 adjacent columns, so R's scattered placement
// costs nothing.  A Z buffer is refilled only after the contraction that
// read its R has completed.  X (+ X_lo) and y have three shared-memory
// stages.  Every wait is bounded.
// ---------------------------------------------------------------------------
constexpr int kTctEpi = 16;                 // epilogue warps: 4 lane quarters x 4 row blocks
constexpr uint32_t kTBhi = 0, kTBlo = 64, kTZ = 128, kTG = 384;
constexpr int kTctStride = 129;             // floats per row of the chain staging tile

template <bool XLO>
struct TctLayout {
  static constexpr int kStages = 3;
  static constexpr int kXStage = (XLO ? 2 : 1) * 32768;   // X [2][128][128 B] (+ X_lo)
  static constexpr int kX = 0;
  static constexpr int kY = kStages * kXStage;            // y - 1/2, [stages][128] float
  static constexpr int kRed = kY + kStages * 512;         // [4 row blocks][128 chains] double
  static constexpr int kCtl = kRed + 4 * 128 * 8;
  static constexpr int kBytes = kCtl + 256;
  // Before the first and after the last TMA load the X stages hold a
  // [128 chains][kTctStride] float tile (states in, gradient out).
  static_assert(128 * kTctStride * 4 <= kY, "chain staging tile must fit the X stages");
  static_assert(kBytes + 1024 <= 232448, "shared memory over the sm_103a limit");
};

struct TctBars {
  uint64_t x_full[3], x_empty[3], z_full[2], r_full[2], zr_free[2], g_done, drain;
};

__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }

// -copysign(w, h): the magnitude of w with the sign of -h.
__device__ __forceinline__ float neg_copysign(float w, float h) {
  return __int_as_float((__float_as_int(w) & 0x7fffffff) |
                        (~__float_as_int(h) & (int)0x80000000));
}

// 32 rows of one chain, two at a time.  With arg = -2 log2(e) |h|,
// t = 2^arg = e^-|z| and u = 1 + t:
//   *sarg += arg (so sum |h| = -sarg / (2 log2 e)),
//   *prod *= u,
//   R = (y - 1/2) - tanh(h)/2 with tanh(|h|)/2 = 1/u - 1/2 (rcp.approx,
//     within one ulp), split into BF16 hi = bf16(R) and lo = bf16(R - hi)
//     (round to nearest), packed as pairs: the gradient contraction's
//     residual correction, R = hi + lo to ~2^-17.
// MASK: rows at or past `nvalid` are padding (X = 0) and leave both sums
// unchanged.
template <bool MASK>
__device__ __forceinline__ void tct_rows(const float (&h)[32], const float* __restrict__ ys,
                                         int nvalid, float2* sarg, float2* prod,
                                         uint32_t (&rp)[16], uint32_t (&rl)[16]) {
  const float2 one = f2(1.f, 1.f), mhalf = f2(-0.5f, -0.5f);
  float2 sa = f2(0.f, 0.f), pr = f2(1.f, 1.f);
#pragma unroll
  for (int g = 0; g < 8; ++g) {
    const float4 yv = *reinterpret_cast<const float4*>(ys + 4 * g);
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      const int j = 4 * g + 2 * e;
      float2 arg = f2(fabsf(h[j]) * kNeg2Log2e, fabsf(h[j + 1]) * kNeg2Log2e);
      float2 u = __fadd2_rn(f2(tc::ex2_approx(arg.x), tc::ex2_approx(arg.y)), one);
      if (MASK) {
        if (j >= nvalid) { arg.x = 0.f; u.x = 1.f; }
        if (j + 1 >= nvalid) { arg.y = 0.f; u.y = 1.f; }
      }
      sa = __fadd2_rn(sa, arg);
      pr = __fmul2_rn(pr, u);
      const float2 w = __fadd2_rn(f2(tc::rcp_approx(u.x), tc::rcp_approx(u.y)), mhalf);
      const float2 ym = e == 0 ? f2(yv.x, yv.y) : f2(yv.z, yv.w);
      const float2 r = __fadd2_rn(ym, f2(neg_copysign(w.x, h[j]), neg_copysign(w.y, h[j + 1])));
      const __nv_bfloat162 rh = __floats2bfloat162_rn(r.x, r.y);
      rp[2 * g + e] = *reinterpret_cast<const uint32_t*>(&rh);
      const float2 rhf = __bfloat1622float2(rh);
      rl[2 * g + e] = pack_bf16x2(r.x - rhf.x, r.y - rhf.y);
    }
  }
  *sarg = sa;
  *prod = pr;
}

template <bool XLO>
__global__ void __launch_bounds__(tc_threads(kTctEpi), 1)
logreg_tct_kernel(const __grid_constant__ CUtensorMap xmap,
                  const __grid_constant__ CUtensorMap xlomap, const float* __restrict__ ym,
                  int N, int D, const float* __restrict__ Q, int ldq,
                  const int* __restrict__ n_dev, int c_base, int c_lim, int grid,
                  double* __restrict__ lpart, float* __restrict__ gpart, int* __restrict__ err) {
  using L = TctLayout<XLO>;
  constexpr int CT = 128;
  constexpr int kThreads = tc_threads(kTctEpi);
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int n = chunk_count(*n_dev, c_base, c_lim);
  const int row_tiles = (N + kRows - 1) / kRows;
  const int S = tc_splits(n, CT, grid, row_tiles);
  const int tiles = (n + CT - 1) / CT;
  if (S == 0 || (int)blockIdx.x >= tiles * S) return;
  const int tile = blockIdx.x % tiles, split = blockIdx.x / tiles;
  const int c0 = tile * CT;
  const int rt_begin = (int)((long long)split * row_tiles / S);
  const int rt_end = (int)((long long)(split + 1) * row_tiles / S);
  const int T = rt_end - rt_begin;
  const int ksteps = (D + 15) >> 4;            // 16-feature K-steps holding data
  const int nkb = (D + 63) >> 6;               // 64-feature blocks of X loaded

  unsigned char* Xs = smem + L::kX;
  float* stage_f = reinterpret_cast<float*>(smem + L::kX);   // [128][kTctStride] staging
  float* Ys = reinterpret_cast<float*>(smem + L::kY);
  double* red = reinterpret_cast<double*>(smem + L::kRed);
  TctBars* bars = reinterpret_cast<TctBars*>(smem + L::kCtl);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + L::kCtl + sizeof(TctBars));
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    for (int i = 0; i < 3; ++i) {
      tc::mbar_init(&bars->x_full[i], 1);
      tc::mbar_init(&bars->x_empty[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      tc::mbar_init(&bars->z_full[i], 1);
      tc::mbar_init(&bars->r_full[i], kTctEpi);
      tc::mbar_init(&bars->zr_free[i], 1);
    }
    tc::mbar_init(&bars->g_done, 1);
    tc::mbar_init(&bars->drain, 1);
    *abort_flag = 0;
    tc::fence_mbar_init();
    tc::prefetch_tmap(&xmap);
    if constexpr (XLO) tc::prefetch_tmap(&xlomap);
  }
  if (warp == 1) tc::tmem_alloc(tmem_slot, 512);
  // Chain states / 2 (coalesced) -> staging tile; the factor 1/2 (exact)
  // makes Z^T hold h = z / 2.
  for (int i = tid; i < CT * 128; i += kThreads) {
    const int cc = i >> 7, d = i & 127;
    stage_f[cc * kTctStride + d] =
        (c0 + cc < n && d < D) ? 0.5f * Q[(size_t)(c0 + cc) * ldq + d] : 0.f;
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  const int quarter = warp & 3;                // TMEM lanes 32*quarter .. (chains)
  const int rblk = (warp - 2) >> 2;            // epilogue: rows / features [32 rblk, +32)
  const uint32_t lane_base = (uint32_t)(quarter * 32) << 16;
  const int c = quarter * 32 + lane;           // chain of this epilogue thread
  if (warp >= 2) {
    // BF16 hi/lo of this chain's 32 features -> TMEM (lane = chain, two
    // features per column).
    const float* src = stage_f + c * kTctStride + rblk * 32;
    uint32_t hi[16], lo[16];
#pragma unroll
    for (int e = 0; e < 16; ++e) {
      const float v0 = src[2 * e], v1 = src[2 * e + 1];
      const __nv_bfloat162 hv = __floats2bfloat162_rn(v0, v1);
      hi[e] = *reinterpret_cast<const uint32_t*>(&hv);
      const float2 hf = __bfloat1622float2(hv);
      lo[e] = pack_bf16x2(v0 - hf.x, v1 - hf.y);
    }
    tc::tmem_st16(tmem + lane_base + kTBhi + rblk * 16, hi);
    tc::tmem_st16(tmem + lane_base + kTBlo + rblk * 16, lo);
    tc::tmem_st_wait();
  }
  // The staging tile is overwritten by TMA next: order these generic-proxy
  // accesses before the async-proxy writes.
  tc::fence_proxy_async_smem();
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();

  if (warp == 0) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      const uint32_t bytes = (uint32_t)nkb * 16384u * (XLO ? 2u : 1u) + 512u;
      int it = 0;
      for (; it < T; ++it) {
        const int s = it % L::kStages;
        if (!wait_or_abort(&bars->x_empty[s], ((uint32_t)(it / L::kStages) & 1) ^ 1,
                           abort_flag)) {
          tc::record_error(err, kTcTimeoutTma);
          *abort_flag = 1;
          break;
        }
        const int r0 = (rt_begin + it) * kRows;
        tc::mbar_arrive_expect_tx(&bars->x_full[s], bytes);
        unsigned char* xs = Xs + s * L::kXStage;
        for (int kb = 0; kb < nkb; ++kb) {
          tc::tma_load_2d(xs + kb * 16384, &xmap, kb * 64, r0, &bars->x_full[s]);
          if constexpr (XLO)
            tc::tma_load_2d(xs + 32768 + kb * 16384, &xlomap, kb * 64, r0, &bars->x_full[s]);
        }
        tc::bulk_load(Ys + s * kRows, ym + r0, 512u, &bars->x_full[s]);
      }
      for (int j = (it > L::kStages ? it - L::kStages : 0); j < it; ++j)
        tc::mbar_wait(&bars->x_full[j % L::kStages], (uint32_t)((j / L::kStages) & 1),
                      kWaitLimitNs);
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      const int nd = ksteps * 16;                                      // N of G^T
      constexpr uint32_t idesc1 = tc::idesc_bf16_f32(128, 128, false, false);
      const uint32_t idesc2 = tc::idesc_bf16_f32(128, nd, false, true);  // MN-major X
      // Shared-memory descriptors are linear in the start address (bits 0-13
      // hold address >> 4; every operand lies below 256 KB, so adding an
      // offset >> 4 never carries out of the field): one base descriptor per
      // major-ness, plus compile-time offsets in the unrolled loops.
      const uint64_t xk = tc::smem_desc_sw128(tc::smem_u32(Xs), 16, 1024);     // K-major
      const uint64_t xmn = tc::smem_desc_sw128(tc::smem_u32(Xs), 16384, 1024); // MN-major
      bool ok = true;
      auto gemm1 = [&](int it) -> bool {
        const int s = it % L::kStages, b = it & 1;
        if (!wait_or_abort(&bars->x_full[s], (uint32_t)(it / L::kStages) & 1, abort_flag))
          return false;
        tc::tc_fence_after();
        const uint64_t xs = xk + (uint64_t)((s * L::kXStage) >> 4);
        const uint32_t tz = tmem + kTZ + b * 128;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          if (k < ksteps) {
            const uint64_t bx = xs + (uint64_t)(((k >> 2) * 16384 + (k & 3) * 32) >> 4);
            tc::mma_bf16_tmem_a(tz, tmem + kTBhi + k * 8, bx, idesc1, k > 0 ? 1u : 0u);
            tc::mma_bf16_tmem_a(tz, tmem + kTBlo + k * 8, bx, idesc1, 1u);
            if constexpr (XLO)
              tc::mma_bf16_tmem_a(tz, tmem + kTBhi + k * 8, bx + (32768 >> 4), idesc1, 1u);
          }
        }
        tc::mma_commit(&bars->z_full[b]);
        return true;
      };
      if (T > 0) ok = gemm1(0);
      if (ok && T > 1) ok = gemm1(1);
      for (int it = 0; it < T && ok; ++it) {
        const int s = it % L::kStages, b = it & 1;
        const uint32_t phase = (uint32_t)(it >> 1) & 1;
        if (!wait_or_abort(&bars->r_full[b], phase, abort_flag)) {
          ok = false;
          break;
        }
        tc::tc_fence_after();
        const uint64_t xs = xmn + (uint64_t)((s * L::kXStage) >> 4);
        const uint32_t tr = tmem + kTZ + b * 128;
#pragma unroll
        for (int ks = 0; ks < kRows / 16; ++ks) {
          // Rows 16 ks .. 16 ks + 15: row block ks / 2, half ks % 2; R_hi at
          // column offset 0 of the block, R_lo at 16.  G^T += R_hi^T X_hi +
          // R_lo^T X_hi (+ R_hi^T X_lo for FP32 data).
          const uint32_t ra = tr + (ks >> 1) * 32 + (ks & 1) * 8;
          const uint64_t bx = xs + (uint64_t)((ks * 2048) >> 4);
          tc::mma_bf16_tmem_a(tmem + kTG, ra, bx, idesc2, (it > 0 || ks > 0) ? 1u : 0u);
          tc::mma_bf16_tmem_a(tmem + kTG, ra + 16, bx, idesc2, 1u);
          if constexpr (XLO)
            tc::mma_bf16_tmem_a(tmem + kTG, ra, bx + (32768 >> 4), idesc2, 1u);
        }
        tc::mma_commit(&bars->x_empty[s]);
        if (it + 2 < T) {
          // Buffer b is refilled only after this contraction has read R.
          tc::mma_commit(&bars->zr_free[b]);
          if (!wait_or_abort(&bars->zr_free[b], phase, abort_flag)) {
            ok = false;
            break;
          }
          tc::tc_fence_after();
          ok = gemm1(it + 2);
        }
      }
      if (ok) {
        tc::mma_commit(&bars->g_done);
      } else {
        tc::record_error(err, kTcTimeoutMma);
        *abort_flag = 1;
      }
      tc::mma_commit(&bars->drain);
      tc::mbar_wait(&bars->drain, 0, kWaitLimitNs);
    }
  } else {
    // ---------------- epilogue (16 warps) ----------------
    // Kahan sum over tiles of sum_r (|h_r| + ln(1 + e^-|z_r|)) for this
    // chain's rows; the linear part sum_r (y_r - 1/2) z_r is added exactly by
    // the reduction.
    constexpr float kArgToAbsH = -1.f / 2.8853900817779268f;   // arg -> |h|
    float acc = 0.f, comp = 0.f;
    bool ok = true;
    for (int it = 0; it < T; ++it) {
      const int s = it % L::kStages, b = it & 1;
      if (!warp_wait(&bars->z_full[b], (uint32_t)(it >> 1) & 1, abort_flag)) {
        ok = false;
        break;
      }
      tc::tc_fence_after();
      const uint32_t tz = tmem + lane_base + kTZ + b * 128 + rblk * 32;
      float h[32];
      tc::tmem_ld32(tz, h);
      tc::tmem_ld_wait();
      // y of this tile: landed with X (already complete; the wait makes the
      // bulk copy's writes visible to this thread).
      if (!warp_wait(&bars->x_full[s], (uint32_t)(it / L::kStages) & 1, abort_flag)) {
        ok = false;
        break;
      }
      const int nvalid = N - ((rt_begin + it) * kRows + rblk * 32);
      const float* ys = Ys + s * kRows + rblk * 32;
      uint32_t rp[16], rl[16];
      float2 sarg, prod;
      if (nvalid >= 32) tct_rows<false>(h, ys, 32, &sarg, &prod, rp, rl);
      else tct_rows<true>(h, ys, nvalid, &sarg, &prod, rp, rl);
      {
        const float sabs = (sarg.x + sarg.y) * kArgToAbsH;
        const float v = fmaf(kLn2, tc::lg2_approx(prod.x * prod.y), sabs) - comp;
        const float t = acc + v;
        comp = (t - acc) - v;
        acc = t;
      }
      // R^T over this warp's 32 Z^T columns (already loaded): hi in the
      // first 16, lo in the last 16.
      tc::tmem_st16(tz, rp);
      tc::tmem_st16(tz + 16, rl);
      tc::tmem_st_wait();
      tc::tc_fence_before();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&bars->r_full[b]);
    }
    if (ok && T > 0) ok = warp_wait(&bars->g_done, 0, abort_flag);
    if (!ok) {
      tc::record_error(err, kTcTimeoutEpilogue);
      *abort_flag = 1;
    } else {
      tc::tc_fence_after();
      // G^T (lane = chain, column = feature) -> staging tile (the X stages
      // are idle: every load has been consumed by the finished MMAs).
      float g[32];
      tc::tmem_ld32(tmem + lane_base + kTG + rblk * 32, g);
      tc::tmem_ld_wait();
      float* dst = stage_f + c * kTctStride + rblk * 32;
#pragma unroll
      for (int j = 0; j < 32; ++j) dst[j] = g[j];
      red[rblk * CT + c] = -((double)acc - (double)comp);
    }
    named_barrier(1, 32 * kTctEpi);
    if (ok) {
      for (int cc = tid - 64; cc < CT; cc += 32 * kTctEpi) {
        const double sum = red[cc] + red[CT + cc] + red[2 * CT + cc] + red[3 * CT + cc];
        if (c0 + cc < n) lpart[(size_t)split * n + c0 + cc] = sum;
      }
      // Coalesced gradient partials: one warp per chain row at a time.
      const int ew = warp - 2;
      for (int cc = ew; cc < CT; cc += kTctEpi) {
        if (c0 + cc >= n) break;
        float* row = gpart + ((size_t)split * n + c0 + cc) * D;
        for (int d = lane; d < D; d += 32) row[d] = stage_f[cc * kTctStride + d];
      }
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem, 512);
  }
}

// ---------------------------------------------------------------------------
// 256 < D <= 512: a cluster of two CTAs shares each (chain tile, row tile).
//
// One CTA cannot hold a 128-row X tile of 512 features (128 KB per stage)
// beside the BF16 hi/lo chain states, so the features are split: CTA p of the
// pair keeps features [256p, 256p + 256) of X and of the states and forms the
// partial Z_p = X[:, F_p] B[:, F_p]^T in its TMEM.  Rows 64p .. 64p+63 belong
// to CTA p: its "send" warps copy the partial of the other 64 rows into the
// peer's exchange buffer (distributed shared memory), its "compute" warps add
// the peer's partial to their own, run the epilogue and write R into both
// CTAs' R tiles.  Each CTA then accumulates G for its own features,
// G_p += X[:, F_p]^T R.  X is read from L2 once per chain tile, as in the
// single-CTA kernel.  Every wait is bounded; a CTA that gives up also sets
// its peer's abort flag.
// ---------------------------------------------------------------------------
constexpr int kPairKB = 4;                  // 64-feature blocks per CTA
constexpr int kPairCT = 64;                 // chains per tile
constexpr int kPairEpi = 16;                // epilogue warps (8 compute + 8 send)
constexpr int kZxStride = kPairCT * 4 + 16; // bytes per exchange row (bank-conflict pad)

struct PairLayout {
  static constexpr int kXStage = kPairKB * 16384;           // [4][128 rows][128 B]
  static constexpr int kBBytes = kPairKB * kPairCT * 128;   // [4][64 chains][128 B]
  static constexpr int kRBuf = 16384;                       // [128 rows][64 chains] BF16
  static constexpr int kX = 0;                              // 2 stages
  static constexpr int kBhi = kX + 2 * kXStage;
  static constexpr int kBlo = kBhi + kBBytes;
  static constexpr int kR = kBlo + kBBytes;
  static constexpr int kZx = kR + kRBuf;                    // [64 rows][kZxStride]
  static constexpr int kCtl = kZx + 64 * kZxStride;
  static constexpr int kBytes = kCtl + 256;
  static_assert(kBytes + 1024 <= 232448, "shared memory over the sm_103a limit");
};

struct PairBars {
  // X stages fill and drain in two halves of 32 KB (features 0-127 and
  // 128-255 of the CTA's 256): the G MMAs of the first 128 features free the
  // first half while those of the second still run, so the refill overlaps
  // the tensor pipe instead of stalling the next tile's Z MMAs.
  uint64_t x_full[2][2], x_empty[2][2];   // [stage][half]
  uint64_t z_full[2], z_empty[2];
  uint64_t zx_full;   // peer's partial for my rows has arrived (8 remote arrivals)
  uint64_t zx_free;   // peer has read what I sent last (8 remote arrivals)
  uint64_t r_full;    // R tile complete (8 local + 8 remote arrivals)
  uint64_t r_free;    // both CTAs' GEMM2 done with R (2 multicast commits)
  uint64_t g_done, drain;
};

__device__ __forceinline__ bool wait_cluster_or_abort(uint64_t* bar, uint32_t parity,
                                                      volatile int* abort_flag) {
  if (tc::mbar_try_wait_cluster(bar, parity)) return true;
  const uint64_t t0 = tc::globaltimer_ns();
  while (true) {
    if (tc::mbar_try_wait_cluster(bar, parity)) return true;
    if (*abort_flag) return false;
    if (tc::globaltimer_ns() - t0 > kWaitLimitNs) return false;
  }
}

__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(tc_threads(kPairEpi), 1)
logreg_tc_pair_kernel(const __grid_constant__ CUtensorMap xmap, const float* __restrict__ y,
                      int N, int D, const float* __restrict__ Q, int ldq,
                      const int* __restrict__ n_dev, int c_base, int c_lim, int pairs,
                      double* __restrict__ lpart, float* __restrict__ gpart,
                      int* __restrict__ err) {
  using L = PairLayout;
  constexpr int CT = kPairCT;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int n = chunk_count(*n_dev, c_base, c_lim);
  const int row_tiles = (N + kRows - 1) / kRows;
  const int S = tc_splits(n, CT, pairs, row_tiles);
  const int tiles = (n + CT - 1) / CT;
  const int pair = blockIdx.x >> 1;
  // Both CTAs of a pair leave together (no cluster barrier is reached).
  if (S == 0 || pair >= tiles * S) return;
  const uint32_t p = tc::cluster_ctarank(), peer = p ^ 1u;
  const int tile = pair % tiles, split = pair / tiles;
  const int c0 = tile * CT;
  const int rt_begin = (int)((long long)split * row_tiles / S);
  const int rt_end = (int)((long long)(split + 1) * row_tiles / S);
  const int T = rt_end - rt_begin;
  const int f0 = 256 * (int)p;                        // first feature of this CTA
  const int fD = min(256, D - f0);                    // features held (>= 1: D > 256)

  unsigned char* Xs = smem + L::kX;
  unsigned char* Bhi = smem + L::kBhi;
  unsigned char* Blo = smem + L::kBlo;
  unsigned char* Rs = smem + L::kR;
  unsigned char* Zx = smem + L::kZx;
  PairBars* bars = reinterpret_cast<PairBars*>(smem + L::kCtl);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + L::kCtl + sizeof(PairBars));
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
  auto abort_both = [&]() {
    *abort_flag = 1;
    tc::st_cluster_u32(tc::map_to_rank(tc::smem_u32((const void*)abort_flag), peer), 1u);
  };

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  float lp_pub = 0.f;   // compute warps, lane j < 16: log-likelihood partial of chain 16 sub + j
  if (tid == 0) {
    for (int i = 0; i < 2; ++i) {
      for (int h = 0; h < 2; ++h) {
        tc::mbar_init(&bars->x_full[i][h], 1);
        tc::mbar_init(&bars->x_empty[i][h], 1);
      }
      tc::mbar_init(&bars->z_full[i], 1);
      tc::mbar_init(&bars->z_empty[i], kPairEpi);
    }
    tc::mbar_init(&bars->zx_full, 8);
    tc::mbar_init(&bars->zx_free, 8);
    tc::mbar_init(&bars->r_full, 16);
    tc::mbar_init(&bars->r_free, 2);
    tc::mbar_init(&bars->g_done, 1);
    tc::mbar_init(&bars->drain, 1);
    *abort_flag = 0;
    tc::fence_mbar_init();
    tc::prefetch_tmap(&xmap);
  }
  if (warp == 1) tc::tmem_alloc(tmem_slot, 256);

  // This CTA's feature half of the chain states / 2 -> BF16 hi/lo, K-major
  // 128-byte-swizzled [4][CT][128 B] (h = z / 2 in the accumulator).
  for (int i = tid; i < CT * kPairKB * 8; i += tc_threads(kPairEpi)) {
    const int c = i / (kPairKB * 8), chunk = i % (kPairKB * 8);
    const int d0 = chunk * 8;
    float v[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const int d = f0 + d0 + e;
      v[e] = (c0 + c < n && d < D) ? 0.5f * Q[(size_t)(c0 + c) * ldq + d] : 0.f;
    }
    uint32_t hi[4], lo[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const __nv_bfloat162 h = __floats2bfloat162_rn(v[2 * e], v[2 * e + 1]);
      hi[e] = *reinterpret_cast<const uint32_t*>(&h);
      const float2 hf = __bfloat1622float2(h);
      lo[e] = pack_bf16x2(v[2 * e] - hf.x, v[2 * e + 1] - hf.y);
    }
    const uint32_t off = (d0 >> 6) * (CT * 128) + tc::sw128_offset(c, d0 & 63);
    *reinterpret_cast<uint4*>(Bhi + off) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
    *reinterpret_cast<uint4*>(Blo + off) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
  }
  tc::fence_proxy_async_smem();
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  // The peer's barriers are initialised before anyone arrives on them.
  tc::cluster_sync();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // ---------------- TMA producer: X[rows, F_p] ----------------
    if (lane == 0) {
      // Half-stage fills in order: fill f is (tile f / 2, half f % 2).
      int nfill = 0;
      bool stop = false;
      for (int it = 0; it < T && !stop; ++it) {
        const int s = it & 1;
        for (int h = 0; h < 2; ++h) {
          if (!wait_or_abort(&bars->x_empty[s][h], ((uint32_t)(it >> 1) & 1) ^ 1, abort_flag)) {
            tc::record_error(err, kTcTimeoutTma);
            abort_both();
            stop = true;
            break;
          }
          tc::mbar_arrive_expect_tx(&bars->x_full[s][h], L::kXStage / 2);
#pragma unroll
          for (int kb = 2 * h; kb < 2 * h + 2; ++kb)
            tc::tma_load_2d(Xs + s * L::kXStage + kb * 16384, &xmap, f0 + kb * 64,
                            (rt_begin + it) * kRows, &bars->x_full[s][h]);
          ++nfill;
        }
      }
      // Let the last fills land before the CTA can exit (each wait bounded).
      for (int f = (nfill > 4 ? nfill - 4 : 0); f < nfill; ++f) {
        const int j = f >> 1, h = f & 1;
        tc::mbar_wait(&bars->x_full[j & 1][h], (uint32_t)((j >> 1) & 1), kWaitLimitNs);
      }
    }
    __syncwarp();
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      constexpr uint32_t idesc1 = tc::idesc_bf16_f32(128, CT, false, false);
      constexpr uint32_t idesc2 = tc::idesc_bf16_f32(128, CT, true, true);
      const uint32_t xs_a = tc::smem_u32(Xs), bhi_a = tc::smem_u32(Bhi);
      const uint32_t blo_a = tc::smem_u32(Blo), rs_a = tc::smem_u32(Rs);
      const uint32_t tg = tmem + 2 * CT;
      const int ksteps = (fD + 15) >> 4;        // K-steps of 16 features holding data
      const int mtiles = (fD + 127) >> 7;       // 128-feature tiles of G
      bool ok = true;
      auto gemm1 = [&](int it) -> bool {
        const int s = it & 1, b = it & 1;
        const uint32_t use = (uint32_t)(it >> 1) & 1;
        if (!wait_or_abort(&bars->z_empty[b], use ^ 1, abort_flag)) return false;
        const uint32_t tz = tmem + b * CT;
        const uint32_t xa = xs_a + s * L::kXStage;
        // Half h holds K-steps 8h .. 8h + 7; a half without data (fD <= 128)
        // is neither waited for nor read.
        for (int h = 0; h < 2 && 8 * h < ksteps; ++h) {
          if (!wait_or_abort(&bars->x_full[s][h], use, abort_flag)) return false;
          tc::tc_fence_after();
#pragma unroll
          for (int kb = 2 * h; kb < 2 * h + 2; ++kb) {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              if (kb * 4 + k >= ksteps) break;
              const uint64_t a = tc::smem_desc_sw128(xa + kb * 16384 + k * 32, 16, 1024);
              const uint64_t bh =
                  tc::smem_desc_sw128(bhi_a + kb * (CT * 128) + k * 32, 16, 1024);
              const uint64_t bl =
                  tc::smem_desc_sw128(blo_a + kb * (CT * 128) + k * 32, 16, 1024);
              tc::mma_bf16(tz, a, bh, idesc1, (kb | k) ? 1u : 0u);
              tc::mma_bf16(tz, a, bl, idesc1, 1u);
            }
          }
        }
        tc::mma_commit(&bars->z_full[b]);
        return true;
      };
      if (T > 0) ok = gemm1(0);
      for (int it = 0; it < T && ok; ++it) {
        if (it + 1 < T) {
          ok = gemm1(it + 1);
          if (!ok) break;
        }
        if (!wait_cluster_or_abort(&bars->r_full, (uint32_t)it & 1, abort_flag)) {
          ok = false;
          break;
        }
        tc::tc_fence_after();
        const uint32_t xa = xs_a + (it & 1) * L::kXStage;
        // M-tile mt reads half mt of the stage; each half is released as soon
        // as the MMAs that read it (and every earlier one) complete.
        for (int mt = 0; mt < mtiles; ++mt) {
#pragma unroll
          for (int ks = 0; ks < kRows / 16; ++ks) {
            const uint64_t a = tc::smem_desc_sw128(xa + mt * 32768 + ks * 2048, 16384, 1024);
            const uint64_t bd = tc::smem_desc_sw128(rs_a + ks * 2048, 16384, 1024);
            tc::mma_bf16(tg + mt * CT, a, bd, idesc2, (it > 0 || ks > 0) ? 1u : 0u);
          }
          tc::mma_commit(&bars->x_empty[it & 1][mt]);
        }
        if (mtiles == 1) tc::mma_commit(&bars->x_empty[it & 1][1]);
        tc::mma_commit_multicast(&bars->r_free, (uint16_t)0x3);
      }
      if (ok) {
        tc::mma_commit(&bars->g_done);
      } else {
        tc::record_error(err, kTcTimeoutMma);
        abort_both();
      }
      tc::mma_commit(&bars->drain);
      tc::mbar_wait(&bars->drain, 0, kWaitLimitNs);
    }
    __syncwarp();
  } else {
    // ---------------- epilogue: 8 compute + 8 send warps ----------------
    // (waits are made warp-uniform so that no lane leaves a loop alone)
    const int quarter = warp & 3;                 // TMEM lanes (rows) 32*quarter ..
    const int sub = (warp - 2) >> 2;              // chains [16 sub, 16 sub + 16)
    const bool compute = (quarter >> 1) == (int)p;  // rows 64p .. 64p+63 are mine
    const uint32_t lane_base = (uint32_t)(quarter * 32) << 16;
    const int r = quarter * 32 + lane;            // row of the tile (TMEM lane)
    const int xrow = (quarter & 1) * 32 + lane;   // row in the 64-row exchange buffer
    const uint32_t zx_peer = tc::map_to_rank(tc::smem_u32(Zx), peer) + xrow * kZxStride + sub * 64;
    const uint32_t r_off = tc::sw128_offset(r, sub * 16);
    const uint32_t r_off8 = tc::sw128_offset(r, sub * 16 + 8);
    const uint32_t r_peer = tc::map_to_rank(tc::smem_u32(Rs), peer);
    const uint32_t zx_full_peer = tc::map_to_rank(tc::smem_u32(&bars->zx_full), peer);
    const uint32_t zx_free_peer = tc::map_to_rank(tc::smem_u32(&bars->zx_free), peer);
    const uint32_t r_full_peer = tc::map_to_rank(tc::smem_u32(&bars->r_full), peer);
    float sacc[16];
#pragma unroll
    for (int c = 0; c < 16; ++c) sacc[c] = 0.f;
    bool ok = true;
    float y_next = 0.f;
    if (compute) {
      const int row0 = rt_begin * kRows + r;
      if (T > 0 && row0 < N) y_next = y[row0];
    }
    for (int it = 0; it < T; ++it) {
      const int b = it & 1;
      const uint32_t ph = (uint32_t)it & 1;
      if (!__all_sync(0xffffffffu, wait_or_abort(&bars->z_full[b], (uint32_t)(it >> 1) & 1, abort_flag))) {
        ok = false;
        break;
      }
      tc::tc_fence_after();
      float h[16];
      tc::tmem_ld16(tmem + b * CT + sub * 16 + lane_base, h);
      tc::tmem_ld_wait();
      tc::tc_fence_before();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&bars->z_empty[b]);
      if (!compute) {
        // Send the partial of the peer's rows.
        if (!__all_sync(0xffffffffu, wait_cluster_or_abort(&bars->zx_free, ph ^ 1, abort_flag))) {
          ok = false;
          break;
        }
#pragma unroll
        for (int j = 0; j < 4; ++j)
          tc::st_cluster_v4(zx_peer + 16 * j,
                            make_uint4(__float_as_uint(h[4 * j]), __float_as_uint(h[4 * j + 1]),
                                       __float_as_uint(h[4 * j + 2]),
                                       __float_as_uint(h[4 * j + 3])));
        // __syncwarp orders every lane's stores before lane 0's arrive, whose
        // release (cluster scope) publishes them to the peer.
        __syncwarp();
        if (lane == 0) tc::mbar_arrive_cluster(zx_full_peer);
        continue;
      }
      // Compute warp: add the peer's partial for this row.
      if (!__all_sync(0xffffffffu, wait_cluster_or_abort(&bars->zx_full, ph, abort_flag))) {
        ok = false;
        break;
      }
      const float4* zx = reinterpret_cast<const float4*>(Zx + xrow * kZxStride + sub * 64);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const float4 v = zx[j];
        h[4 * j] += v.x;
        h[4 * j + 1] += v.y;
        h[4 * j + 2] += v.z;
        h[4 * j + 3] += v.w;
      }
      __syncwarp();
      if (lane == 0) tc::mbar_arrive_cluster(zx_free_peer);
      const int row = (rt_begin + it) * kRows + r;
      const bool valid = row < N;
      const float ym = (valid ? y_next : 0.f) - 0.5f;
      if (it + 1 < T && row + kRows < N) y_next = y[row + kRows];
      uint32_t rp[8] = {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
      if (valid) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const float a = fabsf(h[j]);
          const float t = tc::ex2_approx(a * kNeg2Log2e);       // e^-|z|
          sacc[j] += fmaf(kLn2, tc::lg2_approx(1.f + t), a);
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) rp[j] = residual_bf16x2(h[2 * j], h[2 * j + 1], ym);
      }
      // Both CTAs' GEMM2 of the previous tile must be done with R.
      if (!__all_sync(0xffffffffu, wait_cluster_or_abort(&bars->r_free, ph ^ 1, abort_flag))) {
        ok = false;
        break;
      }
      const uint4 v0 = make_uint4(rp[0], rp[1], rp[2], rp[3]);
      const uint4 v1 = make_uint4(rp[4], rp[5], rp[6], rp[7]);
      *reinterpret_cast<uint4*>(Rs + r_off) = v0;
      *reinterpret_cast<uint4*>(Rs + r_off8) = v1;
      tc::st_cluster_v4(r_peer + r_off, v0);
      tc::st_cluster_v4(r_peer + r_off8, v1);
      tc::fence_proxy_async_smem();
      tc::fence_proxy_async_cluster();
      __syncwarp();
      if (lane == 0) {
        tc::mbar_arrive(&bars->r_full);
        tc::mbar_arrive_cluster(r_full_peer);
      }
    }
    if (ok && T > 0) ok = __all_sync(0xffffffffu, wait_or_abort(&bars->g_done, 0, abort_flag));
    if (!ok) {
      tc::record_error(err, kTcTimeoutEpilogue);
      abort_both();
    } else {
      tc::tc_fence_after();
      // G_p: TMEM lane = feature (of this CTA's half), column = chain.
      for (int mt = 0; mt * 128 < fD; ++mt) {
        const int d = f0 + mt * 128 + quarter * 32 + lane;
        float g[16];
        tc::tmem_ld16(tmem + 2 * CT + mt * CT + sub * 16 + lane_base, g);
        tc::tmem_ld_wait();
        if (d < D) {
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int c = c0 + sub * 16 + j;
            if (c < n) gpart[((size_t)split * n + c) * D + d] = g[j];
          }
        }
      }
    }
    if (compute) {
      // Nonlinear log-likelihood partial of this warp's 32 rows, per chain,
      // into red[p][quarter & 1][chain] of CTA 0 (the exchange buffer is idle
      // after the loop; both CTAs have finished it at the cluster barrier).
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        float v = -sacc[j];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (j == lane) lp_pub = v;
      }
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::cluster_sync();
  if (warp >= 2 && ((warp & 3) >> 1) == (int)p && lane < 16) {
    const int sub = (warp - 2) >> 2;
    const int slot = ((int)p * 2 + (warp & 1)) * CT + sub * 16 + lane;
    const uint32_t dst = tc::map_to_rank(tc::smem_u32(Zx), 0) + slot * 8;
    const double dv = (double)lp_pub;
    asm volatile("st.shared::cluster.f64 [%0], %1;" ::"r"(dst), "d"(dv) : "memory");
  }
  tc::cluster_sync();
  if (p == 0 && !*abort_flag) {
    const double* red = reinterpret_cast<const double*>(Zx);
    for (int c = tid; c < CT; c += tc_threads(kPairEpi)) {
      const double sum = red[c] + red[CT + c] + red[2 * CT + c] + red[3 * CT + c];
      if (c0 + c < n) lpart[(size_t)split * n + c0 + c] = sum;
    }
  }
  if (warp == 1) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem, 256);
  }
}

// FP32 X -> X_hi = bf16(X) and (optionally) X_lo = bf16(X - X_hi), zero-padded
// to Dp features.
__global__ void to_bf16_padded(const float* __restrict__ X, int64_t N, int D, int Dp,
                               __nv_bfloat16* __restrict__ out, __nv_bfloat16* __restrict__ lo) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N * Dp) return;
  const int64_t r = i / Dp;
  const int d = (int)(i % Dp);
  const float v = d < D ? X[r * D + d] : 0.f;
  const __nv_bfloat16 h = __float2bfloat16_rn(v);
  out[i] = h;
  if (lo) lo[i] = __float2bfloat16_rn(v - __bfloat162float(h));
}

__global__ void y_minus_half(const float* __restrict__ y, int64_t N, int64_t padded,
                             float* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < padded) out[i] = i < N ? y[i] - 0.5f : 0.f;
}

__global__ void bf16_pad(const __nv_bfloat16* __restrict__ X, int64_t N, int D, int Dp,
                         __nv_bfloat16* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N * Dp) return;
  const int64_t r = i / Dp;
  const int d = (int)(i % Dp);
  out[i] = d < D ? X[r * D + d] : __float2bfloat16_rn(0.f);
}

// lin[d] = sum_r (y_r - 1/2) X[r][d] in float64, in a fixed order (so every
// target built from the same data gets the same bits): block b sums rows
// [b * chunk, (b + 1) * chunk) into part[b][d], then lin_sum_kernel adds the
// blocks in index order.
__device__ __forceinline__ double as_double(float v) { return (double)v; }
__device__ __forceinline__ double as_double(__nv_bfloat16 v) {
  return (double)__bfloat162float(v);
}

template <class T>
__global__ void lin_partial_kernel(const T* __restrict__ X, const float* __restrict__ y,
                                   int64_t N, int D, int64_t chunk, double* __restrict__ part) {
  const int64_t r0 = (int64_t)blockIdx.x * chunk;
  const int64_t r1 = r0 + chunk < N ? r0 + chunk : N;
  for (int d = threadIdx.x; d < D; d += blockDim.x) {
    double acc = 0.0;
    for (int64_t r = r0; r < r1; ++r) acc += ((double)y[r] - 0.5) * as_double(X[r * D + d]);
    part[(size_t)blockIdx.x * D + d] = acc;
  }
}

__global__ void lin_sum_kernel(const double* __restrict__ part, int nb, int D,
                               double* __restrict__ lin) {
  const int d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= D) return;
  double acc = 0.0;
  for (int b = 0; b < nb; ++b) acc += part[(size_t)b * D + d];
  lin[d] = acc;
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    GBM_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                              cudaEnableDefault, &q));
    if (q != cudaDriverEntryPointSuccess || !p)
      throw CudaError{cudaErrorNotSupported, "cuTensorMapEncodeTiled entry point"};
    fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  return fn;
}

class LogregTc final : public Target {
 public:
  LogregTc(gbm_context* ctx, const void* X, int x_dtype, int64_t n, int64_t d, const float* y,
           float prior_scale)
      : N_(n), D_(d) {
    dim = d;
    kb_ = d <= 128 ? 2 : d <= 256 ? 4 : 8;   // 8: the pair-cluster kernel
    ct_ = kb_ == 2 ? 128 : 64;
    // FP32 data up to 128 features keeps a BF16 residual X_lo (see XLO).
    xlo_ = (x_dtype == 0 && kb_ == 2);
    const int Dp = kb_ * 64;
    xb_.reserve(sizeof(__nv_bfloat16) * (size_t)N_ * Dp);
    if (xlo_) xl_.reserve(sizeof(__nv_bfloat16) * (size_t)N_ * Dp);
    y_.reserve(sizeof(float) * (size_t)N_);
    err_dev_ = ctx->err_dev;
    const int64_t total = N_ * Dp;
    const int tb = 256;
    const int64_t blocks = (total + tb - 1) / tb;
    if (x_dtype == 0)
      to_bf16_padded<<<(unsigned)blocks, tb, 0, ctx->stream>>>(
          static_cast<const float*>(X), N_, (int)D_, Dp, xb_.as<__nv_bfloat16>(),
          xlo_ ? xl_.as<__nv_bfloat16>() : nullptr);
    else
      bf16_pad<<<(unsigned)blocks, tb, 0, ctx->stream>>>(
          static_cast<const __nv_bfloat16*>(X), N_, (int)D_, Dp, xb_.as<__nv_bfloat16>());
    GBM_CUDA(cudaGetLastError());
    GBM_CUDA(cudaMemcpyAsync(y_.ptr, y, sizeof(float) * N_, cudaMemcpyDeviceToDevice,
                             ctx->stream));
    if (kb_ == 2) {
      const int64_t padded = (N_ + kRows - 1) / kRows * kRows;
      ym_.reserve(sizeof(float) * (size_t)padded);
      y_minus_half<<<(unsigned)((padded + 255) / 256), 256, 0, ctx->stream>>>(y, N_, padded,
                                                                              ym_.as<float>());
      GBM_CUDA(cudaGetLastError());
    }
    {
      const int nb = 2 * ctx->num_sms;
      const int64_t chunk = (N_ + nb - 1) / nb;
      DeviceBuffer part;
      part.reserve(sizeof(double) * (size_t)nb * D_);
      lin_.reserve(sizeof(double) * (size_t)D_);
      if (x_dtype == 0)
        lin_partial_kernel<<<nb, 256, 0, ctx->stream>>>(static_cast<const float*>(X), y, N_,
                                                        (int)D_, chunk, part.as<double>());
      else
        lin_partial_kernel<<<nb, 256, 0, ctx->stream>>>(static_cast<const __nv_bfloat16*>(X),
                                                        y, N_, (int)D_, chunk,
                                                        part.as<double>());
      lin_sum_kernel<<<(unsigned)((D_ + 127) / 128), 128, 0, ctx->stream>>>(
          part.as<double>(), nb, (int)D_, lin_.as<double>());
      GBM_CUDA(cudaGetLastError());
      // `part` is freed on scope exit: finish the sum first.
      GBM_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    inv_var_ = 1.f / (prior_scale * prior_scale);
    log_norm_ = -log((double)prior_scale) - 0.5 * log(2.0 * M_PI);
    grid_ = ctx->num_sms;
    if (kb_ == 8) {
      // grid_ counts CTA pairs: as many 2-CTA clusters as can be resident.
      smem_ = PairLayout::kBytes + 1024;
      GBM_CUDA(cudaFuncSetAttribute(logreg_tc_pair_kernel,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_));
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(2 * (ctx->num_sms / 2));
      cfg.blockDim = dim3(tc_threads(kPairEpi));
      cfg.dynamicSmemBytes = smem_;
      int clusters = 0;
      GBM_CUDA(cudaOccupancyMaxActiveClusters(&clusters, logreg_tc_pair_kernel, &cfg));
      grid_ = std::max(1, std::min(ctx->num_sms / 2, clusters));
    }
    encode(&xmap_, xb_.ptr, Dp);
    encode(&xlomap_, xlo_ ? xl_.ptr : xb_.ptr, Dp);
    const int attr = cudaFuncAttributeMaxDynamicSharedMemorySize;
    if (kb_ == 2 && xlo_) {
      smem_ = TctLayout<true>::kBytes + 1024;
      GBM_CUDA(cudaFuncSetAttribute(logreg_tct_kernel<true>, (cudaFuncAttribute)attr,
                                    (int)smem_));
    } else if (kb_ == 2) {
      smem_ = TctLayout<false>::kBytes + 1024;
      GBM_CUDA(cudaFuncSetAttribute(logreg_tct_kernel<false>, (cudaFuncAttribute)attr,
                                    (int)smem_));
    } else if (kb_ == 4) {
      smem_ = TcLayout<4, 64, false>::kBytes + 1024;
      GBM_CUDA(cudaFuncSetAttribute(logreg_tc_kernel<4, 64, 8, false>, (cudaFuncAttribute)attr,
                                    (int)smem_));
    }
  }

  size_t workspace_bytes(int64_t cap) const override {
    const size_t rows = (size_t)grid_ * ct_ + (size_t)cap;
    return rows * sizeof(double) + rows * (size_t)D_ * sizeof(float) + 256;
  }

  void eval(const float* q, int ldq, const int* n_dev, int cap, double* logp, float* grad,
            int ldg, void* ws, cudaStream_t s) override {
    const size_t rows = (size_t)grid_ * ct_ + (size_t)cap;
    double* lpart = static_cast<double*>(ws);
    float* gpart = reinterpret_cast<float*>(lpart + rows);
    const int N = (int)N_, D = (int)D_;
    // One launch covers at most grid_ * ct_ chains (one work item per CTA or
    // CTA pair); larger batches run as consecutive chunks sharing `ws`.
    const int lim = grid_ * ct_;
    for (int base = 0; base < cap; base += lim) {
      const float* qc = q + (size_t)base * ldq;
      // Work items of this launch (CTAs, or CTA pairs for the pair kernel).
      const int g = work_grid(grid_, std::min(lim, cap - base), ct_, N_, kMinSplitRows);
#define GBM_TC_LAUNCH(KB_, CT_, EPI_, XLO_)                                               \
  logreg_tc_kernel<KB_, CT_, EPI_, XLO_><<<g, tc_threads(EPI_), smem_, s>>>(              \
      xmap_, xlomap_, y_.as<float>(), N, D, qc, ldq, n_dev, base, lim, g, lpart, gpart,     \
      err_dev_)
#define GBM_TCT_LAUNCH(XLO_)                                                              \
  logreg_tct_kernel<XLO_><<<g, tc_threads(kTctEpi), smem_, s>>>(                           \
      xmap_, xlomap_, ym_.as<float>(), N, D, qc, ldq, n_dev, base, lim, g, lpart, gpart,     \
      err_dev_)
      if (kb_ == 2 && xlo_) GBM_TCT_LAUNCH(true);
      else if (kb_ == 2) GBM_TCT_LAUNCH(false);
      else if (kb_ == 4) GBM_TC_LAUNCH(4, 64, 8, false);
      else
        logreg_tc_pair_kernel<<<2 * g, tc_threads(kPairEpi), smem_, s>>>(
            xmap_, y_.as<float>(), N, D, qc, ldq, n_dev, base, lim, g, lpart, gpart,
            err_dev_);
#undef GBM_TC_LAUNCH
#undef GBM_TCT_LAUNCH
      GBM_CUDA(cudaGetLastError());
      launch_split_reduce(lpart, gpart, qc, ldq, n_dev, base, lim, std::min(lim, cap - base),
                          ct_, kRows, g, N, D, inv_var_, log_norm_, lin_.as<double>(),
                          logp + base, grad + (size_t)base * ldg, ldg, s);
    }
  }

  int launches_per_eval(int64_t cap) const override {
    return 2 * (int)((cap + (int64_t)grid_ * ct_ - 1) / ((int64_t)grid_ * ct_));
  }
  double flops(int64_t n) const override { return 4.0 * (double)N_ * D_ * n; }
  double bytes(int64_t n) const override {
    return 2.0 * (double)N_ * D_ + 4.0 * N_ + 8.0 * (double)n * D_ + 8.0 * n;
  }

 private:
  int64_t N_, D_;
  int kb_ = 2, ct_ = 128, grid_ = 0;
  size_t smem_ = 0;
  float inv_var_ = 1.f;
  double log_norm_ = 0.0;
  // Tensor map over a BF16 [N][Dp] matrix: boxes of 64 features x 128 rows,
  // 128-byte swizzle, rows past N read as zeros.
  void encode(CUtensorMap* map, void* base, int Dp) {
    cuuint64_t dims[2] = {(cuuint64_t)Dp, (cuuint64_t)N_};
    cuuint64_t strides[1] = {(cuuint64_t)Dp * 2};
    cuuint32_t box[2] = {64, (cuuint32_t)kRows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = encode_tiled()(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, dims, strides,
                                box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw CudaError{cudaErrorInvalidValue, "cuTensorMapEncodeTiled"};
  }

  DeviceBuffer xb_, xl_, y_;
  DeviceBuffer ym_;    // y - 1/2, zero-padded to whole row tiles (chain-major kernel)
  DeviceBuffer lin_;   // X^T (y - 1/2), float64 [D]
  bool xlo_ = false;
  CUtensorMap xlomap_;
  int* err_dev_ = nullptr;
  CUtensorMap xmap_;
};

}  // namespace

std::unique_ptr<Target> make_logreg_tc(gbm_context* ctx, const void* X, int x_dtype, int64_t n,
                                       int64_t d, const float* y, float prior_scale) {
  if (d > 512) return nullptr;
  return std::unique_ptr<Target>(new LogregTc(ctx, X, x_dtype, n, d, y, prior_scale));
}

}  // namespace gbm
