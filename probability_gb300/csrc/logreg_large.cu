// Logistic-regression log-density + gradient above the fused kernels'
// feature limits (FP32 above 256 features, mixed precision above 512): the
// two contractions are plain library GEMMs (cuBLAS, FP32 accumulation) and
// the element-wise work between and after them is this library's own.
//
// Mathematics as in logreg_f32.cu (the inference_gym target,
// spinoffs/inference_gym/inference_gym/targets/logistic_regression.py:92-103,
// distributions/bernoulli.py:126-140):
//   Z = X B^T                       GEMM (N x n), column-major, Z[r + c N]
//   per element: |z|/2 + ln(1 + e^-|z|) summed per chain, R = y - sigmoid(z)
//   G^T = X^T R                     GEMM (D x n) = grad rows [n][D]
//   logp_c = (X^T (y - 1/2)) . q_c - sum_r (|z|/2 + ln(1 + e^-|z|)) + prior
// Mixed precision: X is BF16 (plus a BF16 residual X_lo for FP32 data), the
// states are split into BF16 hi + lo, R into BF16 hi + lo, and the products
// X_hi B_hi^T + X_hi B_lo^T (+ X_lo B_hi^T) and X_hi^T R_hi + X_hi^T R_lo
// (+ X_lo^T R_hi) are accumulated in FP32 -- the residual correction of the
// fused tensor-core kernels.  The hi and lo splits sit side by side as 2n
// columns, so each contraction is one GEMM (plus one for X_lo).  FP32: both
// GEMMs in FP32 (no TF32).
//
// This target evaluates all `cap` states of a call (the GEMM shapes are host
// values): a sampler's inactive rows are computed and ignored.  Every GEMM
// and kernel is launched on the call's stream; the cuBLAS workspace is part
// of the target workspace, so evaluations can be captured in CUDA graphs.
#include <cublas_v2.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <memory>
#include <string>

#include "engine.h"
#include "tc_ptx.cuh"

namespace gbm {
namespace {

constexpr size_t kCublasWs = 32u << 20;   // cuBLAS workspace inside the target workspace
constexpr int kRowBlock = 2048;           // rows per epilogue block
constexpr int kEpiThreads = 256;          // epilogue block size
constexpr int kEpiRows = kRowBlock / kEpiThreads;
constexpr float kNegLog2eL = -1.4426950408889634f;
constexpr float kLn2L = 0.6931471805599453f;

#define GBM_CUBLAS(call)                                                          \
  do {                                                                            \
    cublasStatus_t _s = (call);                                                   \
    if (_s != CUBLAS_STATUS_SUCCESS) throw CudaError{cudaErrorUnknown, #call};    \
  } while (0)

// One cuBLAS handle per host thread (and device): creating a handle can
// synchronise, so it happens once, not per target or evaluation.
cublasHandle_t thread_handle(int device) {
  static thread_local cublasHandle_t h[64] = {};
  if (device < 0 || device >= 64) throw CudaError{cudaErrorInvalidDevice, "device index"};
  if (!h[device]) GBM_CUBLAS(cublasCreate(&h[device]));
  return h[device];
}

size_t align256(size_t b) { return (b + 255) / 256 * 256; }

template <class T> __device__ __forceinline__ T from_float(float v);
template <> __device__ __forceinline__ float from_float<float>(float v) { return v; }
template <> __device__ __forceinline__ __nv_bfloat16 from_float<__nv_bfloat16>(float v) {
  return __float2bfloat16_rn(v);
}

// X [N][D] (float32 or BF16) -> hi [Np][ld] (and lo for FP32 data in the
// mixed form), zero-padded features; ym = y - 1/2.
// Rows N .. Np - 1 (the padding to a multiple of 8 rows) are zero.
template <class TI, class TO>
__global__ void large_pack_kernel(const TI* __restrict__ X, const float* __restrict__ y,
                                  int64_t N, int64_t Np, int D, int ld, TO* __restrict__ hi,
                                  TO* __restrict__ lo, float* __restrict__ ym) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < Np) ym[i] = i < N ? y[i] - 0.5f : 0.f;
  if (i >= Np * ld) return;
  const int64_t r = i / ld;
  const int d = (int)(i - r * ld);
  const float v = (d < D && r < N) ? (float)X[r * D + d] : 0.f;
  const TO h = from_float<TO>(v);
  hi[i] = h;
  if (lo) lo[i] = from_float<TO>(v - (float)h);
}

// lin[d] = sum_r (y_r - 1/2) X[r][d] in float64, fixed order (two passes).
template <class TI>
__global__ void large_lin_partial(const TI* __restrict__ X, const float* __restrict__ y,
                                  int64_t N, int D, int64_t chunk, double* __restrict__ part) {
  const int64_t r0 = (int64_t)blockIdx.x * chunk;
  const int64_t r1 = r0 + chunk < N ? r0 + chunk : N;
  for (int d = threadIdx.x; d < D; d += blockDim.x) {
    double acc = 0.0;
    for (int64_t r = r0; r < r1; ++r) acc += ((double)y[r] - 0.5) * (double)(float)X[r * D + d];
    part[(size_t)blockIdx.x * D + d] = acc;
  }
}

__global__ void large_lin_sum(const double* __restrict__ part, int nb, int D,
                              double* __restrict__ lin) {
  const int d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= D) return;
  double acc = 0.0;
  for (int b = 0; b < nb; ++b) acc += part[(size_t)b * D + d];
  lin[d] = acc;
}

// States q [n][ldq] -> B [n][ld] (hi, and lo in the mixed form), zero-padded.
template <class TO>
__global__ void large_split_states(const float* __restrict__ q, int ldq, int n, int D, int ld,
                                   TO* __restrict__ hi, TO* __restrict__ lo) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)n * ld) return;
  const int64_t c = i / ld;
  const int d = (int)(i - c * ld);
  const float v = d < D ? q[c * ldq + d] : 0.f;
  const TO h = from_float<TO>(v);
  hi[i] = h;
  if (lo) lo[i] = from_float<TO>(v - (float)h);
}

// Over Z [n columns][N rows] (column-major): per (row block, chain) the sum
// of |z|/2 + ln(1 + e^-|z|) (float64 partial) and R = (y - 1/2) - sign(z)
// (1/(1 + e^-|z|) - 1/2) (hi, and lo in the mixed form).
template <class TO>
__global__ void __launch_bounds__(kEpiThreads)
large_epilogue(const float* __restrict__ Z, const float* __restrict__ Zlo,
               const float* __restrict__ ym, int64_t N, int64_t ldz, int n,
               TO* __restrict__ Rhi, TO* __restrict__ Rlo, double* __restrict__ part) {
  __shared__ double red[8];
  const int64_t r0 = (int64_t)blockIdx.x * kRowBlock;
  for (int c = blockIdx.y; c < n; c += gridDim.y) {   // grid.y is capped at 65535
    const float* z = Z + (size_t)c * ldz;
    const float* zl = Zlo ? Zlo + (size_t)c * ldz : nullptr;
    // A thread's kEpiRows rows (stride blockDim): every load is issued before
    // any use, so the block waits for memory once per chain, not per row.
    float zv[kEpiRows], yv[kEpiRows];
#pragma unroll
    for (int k = 0; k < kEpiRows; ++k) {
      const int64_t r = r0 + threadIdx.x + (int64_t)kEpiThreads * k;
      zv[k] = 0.f;
      yv[k] = 0.f;
      if (r < N) {
        zv[k] = zl ? z[r] + zl[r] : z[r];
        yv[k] = ym[r];
      }
    }
    float acc = 0.f;   // this thread's rows in FP32; float64 across threads
#pragma unroll
    for (int k = 0; k < kEpiRows; ++k) {
      const int64_t r = r0 + threadIdx.x + (int64_t)kEpiThreads * k;
      if (r >= ldz) break;
      if (r >= N) {   // padding rows: zero residual, no likelihood term
        Rhi[(size_t)c * ldz + r] = from_float<TO>(0.f);
        if (Rlo) Rlo[(size_t)c * ldz + r] = from_float<TO>(0.f);
        continue;
      }
      const float a = fabsf(zv[k]);
      const float e = tc::ex2_approx(a * kNegLog2eL);
      const float u = 1.f + e;
      acc += fmaf(kLn2L, tc::lg2_approx(u), 0.5f * a);
      const float w = tc::rcp_approx(u) - 0.5f;
      const float rv = zv[k] >= 0.f ? yv[k] - w : yv[k] + w;
      const TO h = from_float<TO>(rv);
      Rhi[(size_t)c * ldz + r] = h;
      if (Rlo) Rlo[(size_t)c * ldz + r] = from_float<TO>(rv - (float)h);
    }
    const double accd = warp_sum((double)acc);
    __syncthreads();                                   // red[] of the previous chain is read
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = accd;
    __syncthreads();
    if (threadIdx.x == 0) {
      double s = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
      part[(size_t)blockIdx.x * n + c] = s;
    }
  }
}

// One warp per chain: log-density from the partials (fixed order), the
// linear term and the prior; gradient G - q / s^2.
__global__ void large_finish(const double* __restrict__ part, int nblk, int n,
                             const float* __restrict__ G, const float* __restrict__ Glo, int ld,
                             const float* __restrict__ q, int ldq,
                             const double* __restrict__ lin, int D, float inv_var,
                             double log_norm, double* __restrict__ logp,
                             float* __restrict__ grad, int ldg) {
  const int c = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (c >= n) return;
  double t = 0.0;
  for (int b = lane; b < nblk; b += 32) t -= part[(size_t)b * n + c];
  for (int d = lane; d < D; d += 32) {
    const float qv = q[(size_t)c * ldq + d];
    t += lin[d] * (double)qv - 0.5 * (double)inv_var * (double)qv * (double)qv;
    const float g = Glo ? G[(size_t)c * ld + d] + Glo[(size_t)c * ld + d] : G[(size_t)c * ld + d];
    grad[(size_t)c * ldg + d] = g - qv * inv_var;
  }
  t = warp_sum(t);
  if (lane == 0) logp[c] = t + (double)D * log_norm;
}

class LogregLarge final : public Target {
 public:
  LogregLarge(gbm_context* ctx, const void* X, int x_dtype, int64_t n, int64_t d, const float* y,
              float prior_scale, bool mixed)
      : N_(n), D_(d), mixed_(mixed), device_(ctx->device) {
    dim = d;
    ld_ = (int)((d + 7) / 8 * 8);
    ldz_ = (N_ + 7) / 8 * 8;
    xlo_ = mixed && x_dtype == 0;
    const size_t el = mixed ? 2 : 4;
    xh_.reserve(el * (size_t)ldz_ * ld_);
    if (xlo_) xl_.reserve(el * (size_t)ldz_ * ld_);
    ym_.reserve(sizeof(float) * (size_t)ldz_);
    const int64_t total = ldz_ * ld_;
    const unsigned blocks = (unsigned)((total + 255) / 256);
    cudaStream_t s = ctx->stream;
    if (mixed && x_dtype == 0)
      large_pack_kernel<float, __nv_bfloat16><<<blocks, 256, 0, s>>>(
          static_cast<const float*>(X), y, N_, ldz_, (int)D_, ld_, xh_.as<__nv_bfloat16>(),
          xl_.as<__nv_bfloat16>(), ym_.as<float>());
    else if (mixed)
      large_pack_kernel<__nv_bfloat16, __nv_bfloat16><<<blocks, 256, 0, s>>>(
          static_cast<const __nv_bfloat16*>(X), y, N_, ldz_, (int)D_, ld_,
          xh_.as<__nv_bfloat16>(), nullptr, ym_.as<float>());
    else
      large_pack_kernel<float, float><<<blocks, 256, 0, s>>>(
          static_cast<const float*>(X), y, N_, ldz_, (int)D_, ld_, xh_.as<float>(), nullptr,
          ym_.as<float>());
    GBM_CUDA(cudaGetLastError());
    {
      const int nb = 2 * ctx->num_sms;
      const int64_t chunk = (N_ + nb - 1) / nb;
      DeviceBuffer part;
      part.reserve(sizeof(double) * (size_t)nb * D_);
      lin_.reserve(sizeof(double) * (size_t)D_);
      if (x_dtype == 0)
        large_lin_partial<<<nb, 256, 0, s>>>(static_cast<const float*>(X), y, N_, (int)D_, chunk,
                                             part.as<double>());
      else
        large_lin_partial<<<nb, 256, 0, s>>>(static_cast<const __nv_bfloat16*>(X), y, N_,
                                             (int)D_, chunk, part.as<double>());
      large_lin_sum<<<(unsigned)((D_ + 127) / 128), 128, 0, s>>>(part.as<double>(), nb,
                                                                 (int)D_, lin_.as<double>());
      GBM_CUDA(cudaGetLastError());
      GBM_CUDA(cudaStreamSynchronize(s));   // `part` is freed on scope exit
    }
    inv_var_ = 1.f / (prior_scale * prior_scale);
    log_norm_ = -log((double)prior_scale) - 0.5 * log(2.0 * M_PI);
  }

  // Column sets: the mixed form stacks the hi and lo state (and residual)
  // splits side by side, so each contraction is one GEMM of 2n columns whose
  // halves are added in FP32 by the epilogue (Z) and the finish (G).
  int sets() const { return mixed_ ? 2 : 1; }

  // [B (sets x n rows) | Z (Np x sets n) | R | G (ld x sets n) | partials |
  //  cuBLAS workspace]
  size_t workspace_bytes(int64_t cap) const override {
    const size_t el = mixed_ ? 2 : 4, w = (size_t)sets() * cap;
    const size_t nblk = (size_t)((N_ + kRowBlock - 1) / kRowBlock);
    return align256(el * w * ld_) + align256(4 * (size_t)ldz_ * w) +
           align256(el * (size_t)ldz_ * w) + align256(4 * w * ld_) + align256(8 * nblk * cap) +
           kCublasWs;
  }

  void eval(const float* q, int ldq, const int*, int cap, double* logp, float* grad, int ldg,
            void* ws, cudaStream_t s) override {
    const size_t el = mixed_ ? 2 : 4;
    const int64_t nblk = (N_ + kRowBlock - 1) / kRowBlock;
    const int n = cap, w = sets() * cap, D = (int)D_;
    unsigned char* p = static_cast<unsigned char*>(ws);
    unsigned char* B = p;          p += align256(el * (size_t)w * ld_);
    float* Z = reinterpret_cast<float*>(p);    p += align256(4 * (size_t)ldz_ * w);
    unsigned char* R = p;          p += align256(el * (size_t)ldz_ * w);
    float* G = reinterpret_cast<float*>(p);    p += align256(4 * (size_t)w * ld_);
    double* part = reinterpret_cast<double*>(p); p += align256(8 * (size_t)nblk * cap);
    void* cws = p;
    cublasHandle_t h = thread_handle(device_);
    GBM_CUBLAS(cublasSetStream(h, s));
    GBM_CUBLAS(cublasSetWorkspace(h, cws, kCublasWs));
    const unsigned sb = (unsigned)(((int64_t)n * ld_ + 255) / 256);
    if (mixed_)
      large_split_states<__nv_bfloat16><<<sb, 256, 0, s>>>(
          q, ldq, n, D, ld_, reinterpret_cast<__nv_bfloat16*>(B),
          reinterpret_cast<__nv_bfloat16*>(B) + (size_t)n * ld_);
    else
      large_split_states<float><<<sb, 256, 0, s>>>(q, ldq, n, D, ld_,
                                                   reinterpret_cast<float*>(B), nullptr);
    GBM_CUDA(cudaGetLastError());
    const cudaDataType_t dt = mixed_ ? CUDA_R_16BF : CUDA_R_32F;
    const float one = 1.f, zero = 0.f;
    // Z = X_hi [B_hi; B_lo]^T (+ X_lo B_hi^T into the first n columns):
    // column-major (Np x w) over the rows padded to a multiple of 8 and the
    // ld_ zero-padded features: every extent the GEMMs see is a multiple of 8
    // elements, so the library picks its aligned tensor-core kernels (with an
    // odd row count it falls back to element-aligned ones, ~15x slower here);
    // the padding of X and of B is zero, so the sums are unchanged.
    const int Kp = ld_, ldz = (int)ldz_;
    auto gemm_z = [&](const void* xa, int cols, const float* beta) {
      GBM_CUBLAS(cublasGemmEx(h, CUBLAS_OP_T, CUBLAS_OP_N, ldz, cols, Kp, &one, xa, dt, ld_, B,
                              dt, ld_, beta, Z, CUDA_R_32F, ldz, CUBLAS_COMPUTE_32F,
                              CUBLAS_GEMM_DEFAULT));
    };
    gemm_z(xh_.ptr, w, &zero);
    if (xlo_) gemm_z(xl_.ptr, n, &one);
    const float* Zlo = mixed_ ? Z + (size_t)n * ldz_ : nullptr;
    const dim3 eg((unsigned)nblk, (unsigned)std::min(n, 65535));
    if (mixed_)
      large_epilogue<__nv_bfloat16><<<eg, kEpiThreads, 0, s>>>(
          Z, Zlo, ym_.as<float>(), N_, ldz_, n, reinterpret_cast<__nv_bfloat16*>(R),
          reinterpret_cast<__nv_bfloat16*>(R) + (size_t)n * ldz_, part);
    else
      large_epilogue<float><<<eg, kEpiThreads, 0, s>>>(Z, nullptr, ym_.as<float>(), N_, ldz_, n,
                                               reinterpret_cast<float*>(R), nullptr, part);
    GBM_CUDA(cudaGetLastError());
    // G^T = X_hi^T [R_hi | R_lo] (+ X_lo^T R_hi into the first n columns):
    // column-major (ld x w) over all ld_ padded features (rows >= D come out
    // zero and are not read) and the Np padded rows (zero residuals).
    auto gemm_g = [&](const void* xa, int cols, const float* beta) {
      GBM_CUBLAS(cublasGemmEx(h, CUBLAS_OP_N, CUBLAS_OP_N, Kp, cols, ldz, &one, xa, dt, ld_, R,
                              dt, ldz, beta, G, CUDA_R_32F, ld_, CUBLAS_COMPUTE_32F,
                              CUBLAS_GEMM_DEFAULT));
    };
    gemm_g(xh_.ptr, w, &zero);
    if (xlo_) gemm_g(xl_.ptr, n, &one);
    large_finish<<<(unsigned)((n + 7) / 8), 256, 0, s>>>(
        part, (int)nblk, n, G, mixed_ ? G + (size_t)n * ld_ : nullptr, ld_, q, ldq,
        lin_.as<double>(), D, inv_var_, log_norm_, logp, grad, ldg);
    GBM_CUDA(cudaGetLastError());
  }

  // split, epilogue, finish + the GEMMs (library kernels, not counted).
  int launches_per_eval(int64_t) const override { return 3; }
  double flops(int64_t n) const override { return 4.0 * (double)N_ * D_ * n; }
  double bytes(int64_t n) const override {
    return (mixed_ ? 2.0 : 4.0) * (double)N_ * D_ + 4.0 * N_ + 8.0 * (double)n * D_ + 8.0 * n;
  }

 private:
  int64_t N_, D_;
  bool mixed_, xlo_ = false;
  int device_ = 0, ld_ = 8;
  int64_t ldz_ = 8;   // leading dimension of Z and R: N rounded up to 8 rows
  float inv_var_ = 1.f;
  double log_norm_ = 0.0;
  DeviceBuffer xh_, xl_, ym_, lin_;
};

}  // namespace

std::unique_ptr<Target> make_logreg_large(gbm_context* ctx, const void* X, int x_dtype, int64_t n,
                                          int64_t d, const float* y, float prior_scale,
                                          bool mixed) {
  if (n >= ((int64_t)1 << 31) || d >= ((int64_t)1 << 20)) return nullptr;   // GEMM dimensions
  return std::unique_ptr<Target>(new LogregLarge(ctx, X, x_dtype, n, d, y, prior_scale, mixed));
}

}  // namespace gbm
