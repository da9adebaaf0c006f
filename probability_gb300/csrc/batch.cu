// Many independent posteriors of uneven dimension in one NUTS sampler.
//
// The members are multivariate normals (MultivariateNormalTriL,
// distributions/mvn_tril.py:44, with the arithmetic of targets_misc.cu) and
// non-centred hierarchical normals (the eight-schools pattern of
// mcmc/eight_schools_hmc.py:41-58).  Their chains are concatenated into one
// ragged population: member t owns chains [c_begin, c_end), and chain c's
// state vector has dim(t) elements at element offset coff[c].  The NUTS
// kernels run on the whole population at once (per-chain step sizes, one
// launch per sampler step for all members), so a leaf of the sampler costs a
// fixed number of launches however many posteriors are in flight.
//
// Gradient evaluation of the active chains is two persistent launches over a
// tile list built on the device each leaf:
//   schedule: for each member, its active chains are a contiguous run of the
//             (sorted) active list; MVN members contribute
//             ceil(active / ct) x ceil(D / 128) tiles, hierarchical members
//             ceil(active / 8) tiles.
//   phase 0:  MVN tiles form u = L^-1 (x - loc) for a block of 128 rows of u
//             and that block's |u|^2; hierarchical tiles do all their work.
//   phase 1:  MVN tiles form grad = -L^-T u for a block of 128 columns; the
//             column-block-0 tile also sums the |u|^2 blocks (fixed order).
// Each CTA walks the list with a stride of the grid, so large and small
// members share the machine in one launch.  The chain-tile width ct (32 or
// 64 chains) is chosen per size class of D by timing both at construction
// (the autotuner).
#include <cuda_runtime.h>

#include <algorithm>
#include <memory>
#include <vector>

#include "engine.h"
#include "gb300_mcmc.h"

namespace gbm {
namespace {

enum BatchFamily : int { kBatchMvn = 1, kBatchHier = 2 };   // the GBM_FAMILY_* values

constexpr int kOB = 128;         // rows / columns of u or grad per MVN tile
constexpr int kKc = 16;          // K chunk
constexpr int kThreads = 256;
constexpr int kHierChains = 8;   // chains per hierarchical tile (a warp each)
constexpr int kClasses = 4;      // size classes of D for the tile autotuner

__host__ __device__ inline int size_class(int d) {
  return d <= 64 ? 0 : d <= 256 ? 1 : d <= 1024 ? 2 : 3;
}

struct BDesc {
  int family, dim, c_begin, c_end;
  long long p_begin;    // first |u|^2 partial of this member
  int ct, nob;          // chain tile and 64-blocks of D (MVN)
  const float* loc;
  const float* linv;
  double log_norm;
  const float* y;
  const float* sigma;
  float mu_scale, tau_scale;
  double hconst;
};

__device__ __forceinline__ int lower_bound_dev(const int* a, int n, int v) {
  int lo = 0, hi = n;
  while (lo < hi) {
    const int m = (lo + hi) >> 1;
    if (a[m] < v) lo = m + 1; else hi = m;
  }
  return lo;
}

// Member index of tile `tile` given the exclusive prefix base[0..T].
__device__ __forceinline__ int member_of(const int* base, int T, int tile) {
  int lo = 0, hi = T;   // base[lo] <= tile < base[hi]
  while (hi - lo > 1) {
    const int m = (lo + hi) >> 1;
    if (base[m] <= tile) lo = m; else hi = m;
  }
  return lo;
}

__global__ void batch_schedule_kernel(const BDesc* __restrict__ d, int T,
                                      const int* __restrict__ act,
                                      const int* __restrict__ act_count, int* __restrict__ a,
                                      int* __restrict__ na, int* __restrict__ t1,
                                      int* __restrict__ t2, int* __restrict__ base1,
                                      int* __restrict__ base2) {
  const int n = *act_count;
  for (int t = threadIdx.x; t < T; t += blockDim.x) {
    const int lo = lower_bound_dev(act, n, d[t].c_begin);
    const int hi = lower_bound_dev(act, n, d[t].c_end);
    const int m = hi - lo;
    a[t] = lo;
    na[t] = m;
    if (d[t].family == kBatchMvn) {
      const int tiles = (m + d[t].ct - 1) / d[t].ct * d[t].nob;
      t1[t] = tiles;
      t2[t] = tiles;
    } else {
      t1[t] = (m + kHierChains - 1) / kHierChains;
      t2[t] = 0;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int s1 = 0, s2 = 0;
    for (int t = 0; t < T; ++t) {
      base1[t] = s1;
      base2[t] = s2;
      s1 += t1[t];
      s2 += t2[t];
    }
    base1[T] = s1;
    base2[T] = s2;
  }
}

struct alignas(16) TileSmem {
  float As[2][kKc][64 + 4];     // [stage][k][chain]
  float Bs[2][kKc][kOB + 4];    // [stage][k][output]
  double red[16][64];
  long long cof[64];
  int cid[64];
};

// One MVN tile: chains act[a0 .. a0 + nc) (nc <= CT) x outputs [o0, o0 + 128).
//   PHASE 0: U[c][o] = sum_{k <= o} (x_c[k] - loc[k]) L^-1[o][k]; |U_c|^2 over
//            the block -> part.
//   PHASE 1: G[c][o] = -sum_{k >= o} U_c[k] L^-1[k][o]; block 0 also writes
//            logp = -1/2 sum of the |U|^2 blocks + log_norm.
// Thread (ty, tx) of the 16 x 16 layout accumulates chains ty*CPT .. +CPT-1
// and outputs tx*4 .. +3 and 64 + tx*4 .. +3 in registers (each K step: one
// shared load of the chains, two conflict-free 16-byte loads of the outputs,
// 8·CPT FMAs).  K chunks of 16 are double-buffered in shared memory: the
// next chunk's global loads are issued into registers before the current
// chunk's FMAs and stored to the other stage after them.
template <int PHASE, int CT>
__device__ void mvn_tile(const BDesc& d, const int* __restrict__ act, int a0, int nc, int ob,
                         const int64_t* __restrict__ coff, const float* __restrict__ X,
                         float* __restrict__ out, double* __restrict__ part,
                         double* __restrict__ logp, TileSmem& sm) {
  constexpr int CPT = CT / 16;                  // chains per thread (4 or 2)
  constexpr int AL = kKc * CT / kThreads;       // A values each thread loads per chunk
  constexpr int BL = kKc * kOB / kThreads;      // B values each thread loads per chunk
  static_assert(AL >= 1 && BL >= 1, "tile loads");
  const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
  const int D = d.dim, o0 = ob * kOB;
  const float* M = d.linv;
  __syncthreads();   // the previous tile is done with shared memory
  if (tid < CT) {
    const int c = tid < nc ? act[a0 + tid] : -1;
    sm.cid[tid] = c;
    sm.cof[tid] = c >= 0 ? coff[c] : 0;
  }
  __syncthreads();
  float acc[CPT][8];
#pragma unroll
  for (int i = 0; i < CPT; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;
  const int k_begin = PHASE == 0 ? 0 : (o0 / kKc) * kKc;
  const int k_end = PHASE == 0 ? min(D, o0 + kOB) : D;
  const int chunks = (k_end - k_begin + kKc - 1) / kKc;
  float ra[AL], rb[BL];
  // Chunk loads: A(k, chain) with k fastest (a chain's state is contiguous);
  // B(k, o) = M[o][k] (phase 0, k fastest) or M[k][o] (phase 1, o fastest).
  auto load = [&](int k0) {
#pragma unroll
    for (int r = 0; r < AL; ++r) {
      const int i = tid + r * kThreads, kk = i % kKc, cc = i / kKc, k = k0 + kk;
      float v = 0.f;
      if (cc < nc && k < D) {
        v = X[sm.cof[cc] + k];
        if (PHASE == 0) v -= d.loc[k];
      }
      ra[r] = v;
    }
#pragma unroll
    for (int r = 0; r < BL; ++r) {
      const int i = tid + r * kThreads;
      if (PHASE == 0) {
        const int kk = i % kKc, oo = i / kKc, k = k0 + kk, o = o0 + oo;
        rb[r] = (o < D && k < D && k <= o) ? M[(size_t)o * D + k] : 0.f;
      } else {
        const int oo = i % kOB, kk = i / kOB, k = k0 + kk, o = o0 + oo;
        rb[r] = (o < D && k < D && k >= o) ? M[(size_t)k * D + o] : 0.f;
      }
    }
  };
  auto store = [&](int st) {
#pragma unroll
    for (int r = 0; r < AL; ++r) {
      const int i = tid + r * kThreads;
      sm.As[st][i % kKc][i / kKc] = ra[r];
    }
#pragma unroll
    for (int r = 0; r < BL; ++r) {
      const int i = tid + r * kThreads;
      if (PHASE == 0)
        sm.Bs[st][i % kKc][i / kKc] = rb[r];
      else
        sm.Bs[st][i / kOB][i % kOB] = rb[r];
    }
  };
  if (chunks > 0) {
    load(k_begin);
    store(0);
  }
  __syncthreads();
  for (int ch = 0; ch < chunks; ++ch) {
    const int st = ch & 1;
    const bool more = ch + 1 < chunks;
    if (more) load(k_begin + (ch + 1) * kKc);
#pragma unroll
    for (int kk = 0; kk < kKc; ++kk) {
      float aa[CPT];
      if (CPT == 4) {
        const float4 a4 = *reinterpret_cast<const float4*>(&sm.As[st][kk][ty * 4]);
        aa[0] = a4.x; aa[1] = a4.y; aa[CPT > 2 ? 2 : 0] = a4.z; aa[CPT > 3 ? 3 : 0] = a4.w;
      } else {
        const float2 a2 = *reinterpret_cast<const float2*>(&sm.As[st][kk][ty * 2]);
        aa[0] = a2.x; aa[1] = a2.y;
      }
      const float4 b0 = *reinterpret_cast<const float4*>(&sm.Bs[st][kk][tx * 4]);
      const float4 b1 = *reinterpret_cast<const float4*>(&sm.Bs[st][kk][64 + tx * 4]);
      const float bb[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
      for (int i = 0; i < CPT; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(aa[i], bb[j], acc[i][j]);
    }
    if (more) store(st ^ 1);
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < CPT; ++i) {
    const int cc = ty * CPT + i;
    double sq = 0.0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int o = o0 + (j < 4 ? tx * 4 + j : 64 + tx * 4 + j - 4);
      if (cc < nc && o < D) {
        const float v = PHASE == 0 ? acc[i][j] : -acc[i][j];
        out[sm.cof[cc] + o] = v;
        sq += (double)v * (double)v;
      }
    }
    if (PHASE == 0) sm.red[tx][cc] = sq;
  }
  if (PHASE == 0) {
    __syncthreads();
    if (tid < nc) {
      double s = 0.0;
      for (int t = 0; t < 16; ++t) s += sm.red[t][tid];
      const int c = sm.cid[tid];
      part[d.p_begin + (long long)(c - d.c_begin) * d.nob + ob] = s;
    }
  } else if (ob == 0 && tid < nc) {
    const int c = sm.cid[tid];
    const double* p = part + d.p_begin + (long long)(c - d.c_begin) * d.nob;
    double s = 0.0;
    for (int t = 0; t < d.nob; ++t) s += p[t];
    logp[c] = -0.5 * s + d.log_norm;   // -1/2 |L^-1 (x - loc)|^2 + normaliser
  }
}

// One hierarchical tile: a warp per chain (targets_misc.cu hier_kernel).
__device__ void hier_tile(const BDesc& d, const int* __restrict__ act, int a0, int nc,
                          const int64_t* __restrict__ coff, const float* __restrict__ Q,
                          double* __restrict__ logp, float* __restrict__ Gout) {
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (w >= nc) return;
  const int c = act[a0 + w];
  const float* x = Q + coff[c];
  float* G = Gout + coff[c];
  const int J = d.dim - 2;
  const float mu = x[0], eta = x[1];
  const float tau = expf(eta);
  float lp = 0.f, gmu = 0.f, geta = 0.f;
  // Four groups per lane per pass: their loads are issued before any use, so
  // a pass waits for memory once instead of four times.
  for (int j0 = lane; j0 < J; j0 += 128) {
    float z[4], sg[4], yy[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int j = j0 + 32 * u;
      z[u] = j < J ? x[2 + j] : 0.f;
      sg[u] = j < J ? d.sigma[j] : 1.f;
      yy[u] = j < J ? d.y[j] : 0.f;
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int j = j0 + 32 * u;
      if (j >= J) break;
      const float res = (yy[u] - (mu + tau * z[u])) / sg[u];
      const float r = res / sg[u];
      lp += -0.5f * z[u] * z[u] - 0.5f * res * res;
      gmu += r;
      geta += r * z[u];
      G[2 + j] = -z[u] + tau * r;
    }
  }
  double lpd = warp_sum((double)lp);
  gmu = warp_sum(gmu);
  geta = warp_sum(geta);
  if (lane == 0) {
    const float t = tau / d.tau_scale;
    lpd += -0.5 * (double)(mu / d.mu_scale) * (double)(mu / d.mu_scale) - log1p((double)t * t) +
           (double)eta + d.hconst;
    logp[c] = lpd;
    G[0] = -mu / (d.mu_scale * d.mu_scale) + gmu;
    G[1] = -2.f * t * t / (1.f + t * t) + 1.f + tau * geta;
  }
}

template <int PHASE>
__global__ void __launch_bounds__(kThreads, 2)
batch_phase_kernel(const BDesc* __restrict__ desc, int T, const int* __restrict__ act,
                   const int* __restrict__ a, const int* __restrict__ na,
                   const int* __restrict__ base, const int64_t* __restrict__ coff,
                   const float* __restrict__ q, float* __restrict__ u, float* __restrict__ grad,
                   double* __restrict__ part, double* __restrict__ logp) {
  __shared__ TileSmem sm;
  const int total = base[T];
  for (int tile = blockIdx.x; tile < total; tile += gridDim.x) {
    const int t = member_of(base, T, tile);
    const BDesc& d = desc[t];
    const int local = tile - base[t];
    if (d.family == kBatchMvn) {
      const int k = local / d.nob, ob = local % d.nob;
      const int a0 = a[t] + k * d.ct;
      const int nc = min(d.ct, na[t] - k * d.ct);
      const float* X = PHASE == 0 ? q : u;
      float* out = PHASE == 0 ? u : grad;
      if (d.ct == 64)
        mvn_tile<PHASE, 64>(d, act, a0, nc, ob, coff, X, out, part, logp, sm);
      else
        mvn_tile<PHASE, 32>(d, act, a0, nc, ob, coff, X, out, part, logp, sm);
    } else if (PHASE == 0) {
      const int a0 = a[t] + local * kHierChains;
      hier_tile(d, act, a0, min(kHierChains, na[t] - local * kHierChains), coff, q, logp, grad);
    }
  }
}

__global__ void iota_kernel(int* idx, int n, int* count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) idx[i] = i;
  if (i == 0) *count = n;
}

class BatchTarget final : public Target {
 public:
  BatchTarget(gbm_context* ctx, const ::gbm_batch_member* m, int64_t count) : ctx_(ctx) {
    T_ = (int)count;
    std::vector<int64_t> coff;
    std::vector<int> cdim;
    hdesc_.resize(T_);
    int64_t elems = 0, parts = 0;
    int chains = 0, dmax = 0;
    for (int t = 0; t < T_; ++t) {
      BDesc& d = hdesc_[t];
      d = BDesc{};
      d.family = m[t].family;
      d.dim = (int)(m[t].family == kBatchMvn ? m[t].dim : m[t].dim + 2);
      d.c_begin = chains;
      d.c_end = chains + (int)m[t].chains;
      d.ct = 64;
      d.nob = (d.dim + kOB - 1) / kOB;
      d.p_begin = parts;
      owned_.emplace_back(new Owned());
      Owned& o = *owned_.back();
      if (d.family == kBatchMvn) {
        o.a.reserve(sizeof(float) * d.dim);
        o.b.reserve(sizeof(float) * (size_t)d.dim * d.dim);
        GBM_CUDA(cudaMemcpyAsync(o.a.ptr, m[t].loc, sizeof(float) * d.dim,
                                 cudaMemcpyDeviceToDevice, ctx->stream));
        GBM_CUDA(cudaMemcpyAsync(o.b.ptr, m[t].scale_tril_inv, sizeof(float) * d.dim * d.dim,
                                 cudaMemcpyDeviceToDevice, ctx->stream));
        d.loc = o.a.as<float>();
        d.linv = o.b.as<float>();
        d.log_norm = m[t].log_normalizer;
        parts += (int64_t)m[t].chains * d.nob;
      } else {
        const int J = d.dim - 2;
        o.a.reserve(sizeof(float) * J);
        o.b.reserve(sizeof(float) * J);
        GBM_CUDA(cudaMemcpyAsync(o.a.ptr, m[t].group_y, sizeof(float) * J,
                                 cudaMemcpyDeviceToDevice, ctx->stream));
        GBM_CUDA(cudaMemcpyAsync(o.b.ptr, m[t].group_sigma, sizeof(float) * J,
                                 cudaMemcpyDeviceToDevice, ctx->stream));
        d.y = o.a.as<float>();
        d.sigma = o.b.as<float>();
        d.mu_scale = m[t].mu_scale;
        d.tau_scale = m[t].tau_scale;
        std::vector<float> hs(J);
        GBM_CUDA(cudaMemcpyAsync(hs.data(), m[t].group_sigma, sizeof(float) * J,
                                 cudaMemcpyDeviceToHost, ctx->stream));
        GBM_CUDA(cudaStreamSynchronize(ctx->stream));
        // Normaliser of the HalfCauchy / Normal priors and the likelihood.
        const double log2pi = log(2.0 * M_PI);
        double c = log(2.0 / M_PI) - log((double)d.mu_scale) - log((double)d.tau_scale) -
                   0.5 * (1.0 + 2.0 * (double)J) * log2pi;
        for (int j = 0; j < J; ++j) c -= log((double)hs[j]);
        d.hconst = c;
      }
      for (int c = 0; c < (int)m[t].chains; ++c) {
        coff.push_back(elems);
        cdim.push_back(d.dim);
        elems += d.dim;
      }
      chains += (int)m[t].chains;
      dmax = std::max(dmax, d.dim);
    }
    C_ = chains;
    E_ = elems;
    dim = dmax;
    coff_.reserve(sizeof(int64_t) * C_);
    cdim_.reserve(sizeof(int) * C_);
    GBM_CUDA(cudaMemcpyAsync(coff_.ptr, coff.data(), sizeof(int64_t) * C_,
                             cudaMemcpyHostToDevice, ctx->stream));
    GBM_CUDA(cudaMemcpyAsync(cdim_.ptr, cdim.data(), sizeof(int) * C_, cudaMemcpyHostToDevice,
                             ctx->stream));
    desc_.reserve(sizeof(BDesc) * T_);
    u_.reserve(sizeof(float) * (size_t)E_);
    part_.reserve(sizeof(double) * (size_t)std::max<int64_t>(parts, 1));
    sched_.reserve(sizeof(int) * (size_t)(6 * (T_ + 1)));
    all_.reserve(sizeof(int) * (size_t)(C_ + 1));
    // Persistent CTAs: as many as are resident at once (a second wave would
    // start its share of the tile list late).
    int occ0 = 0, occ1 = 0;
    GBM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ0, batch_phase_kernel<0>,
                                                           kThreads, 0));
    GBM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ1, batch_phase_kernel<1>,
                                                           kThreads, 0));
    grid_ = std::max(1, std::min(occ0, occ1)) * ctx->num_sms;
    upload();
    GBM_CUDA(cudaStreamSynchronize(ctx->stream));
    autotune();
  }

  size_t workspace_bytes(int64_t) const override { return 256; }
  const int64_t* ragged_offsets() const override { return coff_.as<int64_t>(); }
  const int* ragged_dims() const override { return cdim_.as<int>(); }
  int64_t ragged_chains() const override { return C_; }
  int64_t ragged_elements() const override { return E_; }
  int launches_per_eval(int64_t) const override { return 3; }

  // All chains (the direct log_prob_and_grad call): q, grad ragged.
  void eval(const float* q, int, const int*, int, double* logp, float* grad, int, void*,
            cudaStream_t s) override {
    int* idx = all_.as<int>();
    iota_kernel<<<(C_ + 255) / 256, 256, 0, s>>>(idx, C_, idx + C_);
    GBM_CUDA(cudaGetLastError());
    eval_active(q, idx, idx + C_, logp, grad, nullptr, s);
  }

  void eval_active(const float* q, const int* act, const int* act_count, double* logp,
                   float* grad, void*, cudaStream_t s) override {
    int* w = sched_.as<int>();
    const int T1 = T_ + 1;
    int *a = w, *na = w + T1, *t1 = w + 2 * T1, *t2 = w + 3 * T1, *b1 = w + 4 * T1,
        *b2 = w + 5 * T1;
    const BDesc* d = desc_.as<BDesc>();
    batch_schedule_kernel<<<1, 1024, 0, s>>>(d, T_, act, act_count, a, na, t1, t2, b1, b2);
    batch_phase_kernel<0><<<grid_, kThreads, 0, s>>>(d, T_, act, a, na, b1, coff_.as<int64_t>(),
                                                     q, u_.as<float>(), grad,
                                                     part_.as<double>(), logp);
    batch_phase_kernel<1><<<grid_, kThreads, 0, s>>>(d, T_, act, a, na, b2, coff_.as<int64_t>(),
                                                     q, u_.as<float>(), grad,
                                                     part_.as<double>(), logp);
    GBM_CUDA(cudaGetLastError());
  }

  double flops(int64_t) const override {
    double f = 0.0;
    for (const BDesc& d : hdesc_) {
      const double n = d.c_end - d.c_begin;
      f += d.family == kBatchMvn ? 2.0 * d.dim * (double)d.dim * n : 10.0 * (d.dim - 2) * n;
    }
    return f;
  }
  double bytes(int64_t) const override {
    double b = 0.0;
    for (const BDesc& d : hdesc_) {
      const double n = d.c_end - d.c_begin;
      b += d.family == kBatchMvn ? 4.0 * d.dim * (double)d.dim + 8.0 * n * d.dim + 8.0 * n
                                 : 8.0 * (d.dim - 2) + 8.0 * n * d.dim + 8.0 * n;
    }
    return b;
  }

  // Chain-tile width chosen for each size class of D (0 if the class is empty).
  void schedule(int32_t* ct) const {
    for (int k = 0; k < kClasses; ++k) ct[k] = chosen_[k];
  }

 private:
  struct Owned {
    DeviceBuffer a, b;
  };

  void upload() {
    GBM_CUDA(cudaMemcpyAsync(desc_.ptr, hdesc_.data(), sizeof(BDesc) * T_,
                             cudaMemcpyHostToDevice, ctx_->stream));
  }

  // For each size class of D: time a full evaluation of every chain with
  // that class's MVN tiles at 32 and at 64 chains and keep the faster.
  void autotune() {
    cudaStream_t s = ctx_->stream;
    double* lp = nullptr;
    float* g = nullptr;
    DeviceBuffer qb, lb, gb;
    qb.reserve(sizeof(float) * (size_t)E_);
    lb.reserve(sizeof(double) * (size_t)C_);
    gb.reserve(sizeof(float) * (size_t)E_);
    GBM_CUDA(cudaMemsetAsync(qb.ptr, 0, sizeof(float) * (size_t)E_, s));
    lp = lb.as<double>();
    g = gb.as<float>();
    cudaEvent_t e0, e1;
    GBM_CUDA(cudaEventCreate(&e0));
    GBM_CUDA(cudaEventCreate(&e1));
    for (int k = 0; k < kClasses; ++k) {
      chosen_[k] = 0;
      bool any = false;
      for (const BDesc& d : hdesc_) any |= d.family == kBatchMvn && size_class(d.dim) == k;
      if (!any) continue;
      float best = 1e30f;
      for (int ct : {32, 64}) {
        for (BDesc& d : hdesc_)
          if (d.family == kBatchMvn && size_class(d.dim) == k) d.ct = ct;
        upload();
        eval(qb.as<float>(), 0, nullptr, 0, lp, g, 0, nullptr, s);   // warm-up
        GBM_CUDA(cudaEventRecord(e0, s));
        for (int r = 0; r < 3; ++r) eval(qb.as<float>(), 0, nullptr, 0, lp, g, 0, nullptr, s);
        GBM_CUDA(cudaEventRecord(e1, s));
        GBM_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        GBM_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best) {
          best = ms;
          chosen_[k] = ct;
        }
      }
      for (BDesc& d : hdesc_)
        if (d.family == kBatchMvn && size_class(d.dim) == k) d.ct = chosen_[k];
    }
    upload();
    GBM_CUDA(cudaStreamSynchronize(s));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
  }

  gbm_context* ctx_;
  int T_ = 0, C_ = 0, grid_ = 0;
  int64_t E_ = 0;
  int chosen_[kClasses] = {0, 0, 0, 0};
  std::vector<BDesc> hdesc_;
  std::vector<std::unique_ptr<Owned>> owned_;
  DeviceBuffer desc_, coff_, cdim_, u_, part_, sched_, all_;
};

}  // namespace

std::unique_ptr<Target> make_batch(gbm_context* ctx, const ::gbm_batch_member* m,
                                   int64_t count) {
  return std::unique_ptr<Target>(new BatchTarget(ctx, m, count));
}

bool batch_schedule(const Target* t, int32_t* ct) {
  const auto* b = dynamic_cast<const BatchTarget*>(t);
  if (!b) return false;
  b->schedule(ct);
  return true;
}

}  // namespace gbm
