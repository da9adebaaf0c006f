// HMC, NUTS and dual-averaging kernels plus their host-side orchestration.
//
// Chains live in chain-major [C][D] float32 arrays; log-densities, energies,
// NUTS log-weights and energy-difference sums are float64.  Each per-chain
// kernel runs one warp per chain with lanes striding over D.
//
// NUTS follows the reference's unrolled iterative formulation
// (tensorflow_probability/python/mcmc/nuts.py:321-1102): multinomial
// sampling, generalised U-turn criterion with the precomputed write/read slot
// tables.  Unlike the reference's lock-step batch, only chains whose subtree
// is still growing are evaluated: after every leaf the active chains are
// compacted into a dense batch, so the gradient kernels never spend work on
// finished chains.  Per-chain results are unchanged by this (a finished
// chain's outputs are frozen in the reference, nuts.py:829-933), and draws
// are addressed by (chain, depth, leaf) so compaction does not shift them.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "rng.cuh"
#include "samplers.h"

namespace gbm {

constexpr int kWarpsPerBlock = 8;

static inline int warp_blocks(int64_t n) {
  return (int)((n + kWarpsPerBlock - 1) / kWarpsPerBlock);
}

__device__ __forceinline__ int warp_id() {
  return (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
}

__device__ __forceinline__ float eps_of(const float* eps, int per_chain, int c) {
  return per_chain ? eps[c] : eps[0];
}

// Layout helpers (uniform or ragged, see NutsDev).
__device__ __forceinline__ size_t voff(const NutsDev& w, int c) {
  return w.ragged ? (size_t)w.coff[c] : (size_t)c * w.D;
}
__device__ __forceinline__ int vdim(const NutsDev& w, int c) {
  return w.ragged ? w.cdim[c] : w.D;
}
// Start of U-turn slot i of chain c.
__device__ __forceinline__ size_t soff(const NutsDev& w, int c, int i) {
  return w.ragged ? (size_t)w.coff[c] * w.slots + (size_t)i * w.cdim[c]
                  : ((size_t)c * w.slots + i) * w.D;
}
// Start of chain c (at batch position j) in the gradient batch qw / gw.
__device__ __forceinline__ size_t boff(const NutsDev& w, int c, int j) {
  return w.ragged ? (size_t)w.coff[c] : (size_t)j * w.D;
}
__device__ __forceinline__ int lwi(const NutsDev& w, int c, int j) { return w.ragged ? c : j; }
// Inverse mass of element d of the chain whose vector starts at o (1: identity).
__device__ __forceinline__ float imass(const NutsDev& w, size_t o, int d) {
  return w.inv_mass ? (w.im_per_chain ? w.inv_mass[o + d] : w.inv_mass[d]) : 1.f;
}

// --------------------------------------------------------------------------
// Active-chain compaction: idx[0..count) = chains with (flags & bit), sorted.
// --------------------------------------------------------------------------
__global__ void build_active_kernel(const uint8_t* __restrict__ flags, uint8_t bit, int C,
                                    int* __restrict__ idx, int* __restrict__ count) {
  __shared__ int warp_tot[32];
  __shared__ int base_s;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  if (tid == 0) base_s = 0;
  __syncthreads();
  for (int start = 0; start < C; start += blockDim.x) {
    const int c = start + tid;
    const bool on = c < C && (flags[c] & bit);
    const unsigned m = __ballot_sync(0xffffffffu, on);
    if (lane == 0) warp_tot[w] = __popc(m);
    __syncthreads();
    if (w == 0) {
      int v = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0;
      int incl = v;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
      }
      if (lane < (int)(blockDim.x >> 5)) warp_tot[lane] = incl - v;  // exclusive
    }
    __syncthreads();
    const int base = base_s;
    if (on) idx[base + warp_tot[w] + __popc(m & ((1u << lane) - 1u))] = c;
    __syncthreads();
    if (tid == blockDim.x - 1) {
      const unsigned mm = m;  // last warp's ballot
      base_s = base + warp_tot[w] + __popc(mm);
    }
    __syncthreads();
  }
  if (tid == 0) *count = base_s;
}

cudaStream_t& alloc_stream() {
  static thread_local cudaStream_t s = nullptr;
  return s;
}

__global__ void set_count_kernel(int* count, int n) { *count = n; }
__global__ void set_key_kernel(uint2* keyp, uint2 key) { *keyp = key; }

void set_count(int* count, int n, cudaStream_t s) {
  set_count_kernel<<<1, 1, 0, s>>>(count, n);
  GBM_CUDA(cudaGetLastError());
}

// Large batches: per-block counts, then an order-preserving scatter (each
// block adds the counts of the blocks before it), so the list stays sorted.
constexpr int kActBlock = 1024;

__global__ void active_block_count_kernel(const uint8_t* __restrict__ flags, uint8_t bit, int C,
                                          int* __restrict__ blk) {
  const int c = blockIdx.x * kActBlock + threadIdx.x;
  const int n = __syncthreads_count(c < C && (flags[c] & bit));
  if (threadIdx.x == 0) blk[blockIdx.x] = n;
}

__global__ void active_block_scatter_kernel(const uint8_t* __restrict__ flags, uint8_t bit, int C,
                                            const int* __restrict__ blk, int* __restrict__ idx,
                                            int* __restrict__ count) {
  __shared__ int warp_tot[32];
  __shared__ int base_s;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int nw = kActBlock >> 5;
  int part = 0;
  for (int b = tid; b < (int)blockIdx.x; b += kActBlock) part += blk[b];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  if (lane == 0) warp_tot[w] = part;
  __syncthreads();
  if (tid == 0) {
    int sum = 0;
    for (int i = 0; i < nw; ++i) sum += warp_tot[i];
    base_s = sum;
  }
  __syncthreads();
  const int base = base_s;
  const int c = blockIdx.x * kActBlock + tid;
  const bool on = c < C && (flags[c] & bit);
  const unsigned m = __ballot_sync(0xffffffffu, on);
  __syncthreads();   // everyone has read warp_tot's block sums
  if (lane == 0) warp_tot[w] = __popc(m);
  __syncthreads();
  if (w == 0) {
    const int v = lane < nw ? warp_tot[lane] : 0;
    int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    if (lane < nw) warp_tot[lane] = incl - v;   // exclusive
  }
  __syncthreads();
  if (on) idx[base + warp_tot[w] + __popc(m & ((1u << lane) - 1u))] = c;
  if (tid == 0 && blockIdx.x == gridDim.x - 1) *count = base + blk[blockIdx.x];
}

static int active_launches(int C) { return C <= 2 * kActBlock ? 1 : 2; }

static void build_active(const NutsDev& d, uint8_t bit, cudaStream_t s) {
  if (d.C <= 2 * kActBlock) {
    build_active_kernel<<<1, 1024, 0, s>>>(d.flags, bit, d.C, d.act_idx, d.act_count);
  } else {
    const int nb = (d.C + kActBlock - 1) / kActBlock;
    active_block_count_kernel<<<nb, kActBlock, 0, s>>>(d.flags, bit, d.C, d.act_blk);
    active_block_scatter_kernel<<<nb, kActBlock, 0, s>>>(d.flags, bit, d.C, d.act_blk,
                                                         d.act_idx, d.act_count);
  }
  GBM_CUDA(cudaGetLastError());
}

// --------------------------------------------------------------------------
// NUTS kernels
// --------------------------------------------------------------------------
// The kernels below are thin launches of per-chain bodies (one warp, or one
// thread, per chain) shared by the lock-step transition (all chains at the
// same depth and leaf) and the free-running loop (every chain at its own).

// Momentum draw and trajectory start of chain c from (q, l, g)
// (nuts.py:512-539); q may alias cand_q (the free-running loop starts each
// transition from the previous one's result).
__device__ void nuts_chain_init(const NutsDev& w, int c, int lane, const float* q, const double* l,
                                const float* g, float eps_c, uint2 key) {
  const int D = vdim(w, c);
  const size_t o = voff(w, c);
  const uint32_t site = draw_site(kDrawMomentum, 0, 0);
  float kin_l = 0.f;   // this lane's share of |p|^2 (FP32); summed across lanes in FP64
  for (int d = lane; d < D; d += 32) {
    const float im = imass(w, o, d);
    // p ~ N(0, M): z / sqrt(M^-1) (preconditioned_nuts.py momentum draw)
    const float p = w.inv_mass ? draw_normal(key, site, (uint32_t)(o + d)) / sqrtf(im)
                               : draw_normal(key, site, (uint32_t)(o + d));
    const float qd = q[o + d], gd = g[o + d];
    w.end_q[0][o + d] = qd; w.end_q[1][o + d] = qd;
    w.end_p[0][o + d] = p;  w.end_p[1][o + d] = p;
    w.end_g[0][o + d] = gd; w.end_g[1][o + d] = gd;
    w.cand_q[o + d] = qd;   w.cand_g[o + d] = gd;
    w.mom_sum[o + d] = p;
    kin_l = fmaf(p * im, p, kin_l);     // p^T M^-1 p
  }
  const double kin = warp_sum((double)kin_l);
  if (lane == 0) {
    const double lc = l[c];
    const double e0 = lc - 0.5 * kin;   // nuts.py:1085-1102 (negative energy)
    w.end_l[0][c] = lc; w.end_l[1][c] = lc;
    w.cand_l[c] = lc; w.cand_e[c] = e0; w.cand_w[c] = 0.0;
    w.e0[c] = e0; w.eds[c] = 0.0; w.lf[c] = 0; w.tree_depth[c] = 0;
    w.flags[c] = kCont | kNotDiv;
    w.eps[c] = eps_c;
  }
}

__global__ void nuts_init_kernel(NutsDev w, const float* __restrict__ q,
                                 const double* __restrict__ l, const float* __restrict__ g,
                                 const float* __restrict__ eps_in, int eps_per_chain, uint2 key) {
  const int c = warp_id(), lane = threadIdx.x & 31;
  if (c >= w.C) return;
  nuts_chain_init(w, c, lane, q, l, g, eps_of(eps_in, eps_per_chain, c), key);
}

// Start of a tree depth for chain c (one thread): direction draw and the
// subtree's initial state (nuts.py:551-558, 727-731).
__device__ void nuts_chain_depth_begin(const NutsDev& w, int c, uint2 key, int depth) {
  uint8_t f = w.flags[c];
  if (!(f & kCont)) {
    w.flags[c] = f & (uint8_t)~(kSubCont | kForward);
    return;
  }
  const int fwd = draw_direction(key, (uint32_t)depth, (uint32_t)c);   // nuts.py:551-558
  f = (f & (uint8_t)~(kForward | kSubNotDiv)) | kSubCont | (fwd ? kForward : 0) |
      ((f & kNotDiv) ? kSubNotDiv : 0);
  w.flags[c] = f;
  w.sub_w[c] = -INFINITY;               // nuts.py:727-731
  w.sub_eds[c] = 0.0;
  w.sub_lf[c] = 0;
  w.tree_depth[c] += 1;
}

__global__ void nuts_depth_begin_kernel(NutsDev w, uint2 key, int depth) {
  if (blockIdx.x == 0 && threadIdx.x == 0) *w.any_cont = 0;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= w.C) return;
  nuts_chain_depth_begin(w, c, key, depth);
}

__device__ void nuts_chain_zero_cumsum(const NutsDev& w, int c, int lane) {
  const size_t o = voff(w, c);
  const int D = vdim(w, c);
  for (int d = lane; d < D; d += 32) w.cumsum[o + d] = 0.f;
}

__global__ void nuts_zero_cumsum_kernel(NutsDev w) {
  const int c = warp_id(), lane = threadIdx.x & 31;
  if (c >= w.C || !(w.flags[c] & kSubCont)) return;
  nuts_chain_zero_cumsum(w, c, lane);
}

// Half kick + drift of chain c (batch position j); writes the dense batch qw.
// leapfrog_integrator.py:280-286 (half kick) and :330-334 (drift).
__device__ void nuts_chain_leaf_pre(const NutsDev& w, int c, int j, int lane) {
  const int side = (w.flags[c] & kForward) ? 1 : 0;
  const float e = (side ? 1.f : -1.f) * w.eps[c];
  const float he = 0.5f * e;
  const size_t o = voff(w, c), oj = boff(w, c, j);
  const int D = vdim(w, c);
  float* P = w.end_p[side];
  float* Q = w.end_q[side];
  const float* G = w.end_g[side];
  // Four elements per pass with every load issued before the stores (the
  // arrays may alias as far as the compiler knows, so it would not hoist
  // them itself); the arithmetic per element is the same as the tail's.
  int d = lane;
  for (; d + 96 < D; d += 128) {
    float pv[4], gv[4], qv[4], iv[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const size_t x = o + d + 32 * u;
      pv[u] = P[x];
      gv[u] = G[x];
      qv[u] = Q[x];
      iv[u] = imass(w, o, d + 32 * u);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const size_t x = o + d + 32 * u;
      const float ph = pv[u] + he * gv[u];
      const float qn = qv[u] + e * (ph * iv[u]);
      P[x] = ph;
      Q[x] = qn;
      w.qw[oj + d + 32 * u] = qn;
    }
  }
  for (; d < D; d += 32) {
    const float ph = P[o + d] + he * G[o + d];
    const float qn = Q[o + d] + e * (ph * imass(w, o, d));   // drift by the velocity
    P[o + d] = ph;
    Q[o + d] = qn;
    w.qw[oj + d] = qn;
  }
}

__global__ void nuts_leaf_pre_kernel(NutsDev w) {
  const int j = warp_id(), lane = threadIdx.x & 31;
  if (j >= *w.act_count) return;
  nuts_chain_leaf_pre(w, w.act_idx[j], j, lane);
}

// Between the unrolled leapfrog steps of one leaf: full kick then drift.
__global__ void nuts_leaf_mid_kernel(NutsDev w) {
  const int j = warp_id(), lane = threadIdx.x & 31;
  if (j >= *w.act_count) return;
  const int c = w.act_idx[j];
  const int side = (w.flags[c] & kForward) ? 1 : 0;
  const float e = (side ? 1.f : -1.f) * w.eps[c];
  const size_t o = voff(w, c), oj = boff(w, c, j);
  const int D = vdim(w, c);
  for (int d = lane; d < D; d += 32) {
    const float ph = w.end_p[side][o + d] + e * w.gw[oj + d];
    const float qn = w.end_q[side][o + d] + e * (ph * imass(w, o, d));
    w.end_p[side][o + d] = ph;
    w.end_q[side][o + d] = qn;
    w.qw[oj + d] = qn;
  }
}

// Final kick, slot bookkeeping, U-turn checks, energy, multinomial leaf
// sampling: _loop_build_sub_tree (nuts.py:793-946) and
// has_not_u_turn_at_all_index (nuts.py:949-984).
__device__ void nuts_chain_leaf_post(const NutsDev& w, int c, int j, int lane, uint2 key,
                                     int depth, int leaf, int wslot, int r0, int r1,
                                     double max_energy_diff) {
  const int D = vdim(w, c);
  const uint8_t f = w.flags[c];
  const int side = (f & kForward) ? 1 : 0;
  const float e = (side ? 1.f : -1.f) * w.eps[c];
  const float he = 0.5f * e;
  const size_t o = voff(w, c), oj = boff(w, c, j);
  float* P = w.end_p[side];
  float* Gs = w.end_g[side];
  float kin_l = 0.f;
  // Four elements per pass, loads first (as in the half kick above); the
  // tail loop is the per-element form.  kin_l accumulates in element order.
  int d = lane;
  for (; d + 96 < D; d += 128) {
    float g2v[4], pv[4], csv[4], imv[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int x = d + 32 * u;
      g2v[u] = w.gw[oj + x];
      pv[u] = P[o + x];
      csv[u] = w.cumsum[o + x];
      imv[u] = imass(w, o, x);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int x = d + 32 * u;
      const float p2 = (pv[u] + e * g2v[u]) - he * g2v[u];
      P[o + x] = p2;
      Gs[o + x] = g2v[u];
      w.cumsum[o + x] = csv[u] + p2;
      if (wslot >= 0) {
        const size_t so = soff(w, c, wslot) + x;
        w.slot_p[so] = p2 * imv[u];
        w.slot_cs[so] = csv[u];
      }
      kin_l = fmaf(p2 * imv[u], p2, kin_l);
    }
  }
  for (; d < D; d += 32) {
    const float g2 = w.gw[oj + d];
    const float p2 = (P[o + d] + e * g2) - he * g2;   // leapfrog_integrator.py:345-349,:304-309
    P[o + d] = p2;
    Gs[o + d] = g2;
    const float csp = w.cumsum[o + d];
    const float cs = csp + p2;                          // nuts.py:827-828
    w.cumsum[o + d] = cs;
    const float im = imass(w, o, d);
    if (wslot >= 0) {                                   // nuts.py:857-869
      const size_t so = soff(w, c, wslot) + d;
      w.slot_p[so] = p2 * im;                           // velocity (preconditioned_nuts.py:877-885)
      w.slot_cs[so] = csp;
    }
    kin_l = fmaf(p2 * im, p2, kin_l);
  }
  const double kin = warp_sum((double)kin_l);
  __syncwarp();
  // Within-subtree U-turn over the read range (reads never hit wslot: a leaf
  // that ends subtrees writes only the dummy slot, which is skipped).  The
  // dot products are FP32, the state's type, as in the reference (GB300's
  // FP64 pipe is narrow); the slot loop stays rolled to keep registers (and
  // occupancy over tens of thousands of chains) reasonable.
  bool no_uturn = true;
#pragma unroll 1
  for (int i = r0; i < r1; ++i) {
    float dl = 0.f, dr = 0.f;
    const size_t so = soff(w, c, i);
    for (int d = lane; d < D; d += 32) {
      const float diff = w.cumsum[o + d] - w.slot_cs[so + d];
      dl = fmaf(diff, w.slot_p[so + d], dl);
      dr = fmaf(diff, P[o + d] * imass(w, o, d), dr);   // velocity
    }
    dl = warp_sum(dl);
    dr = warp_sum(dr);
    no_uturn = no_uturn && (dl >= 0.f) && (dr >= 0.f);
  }
  const double l2 = w.lw[lwi(w, c, j)];
  double energy = l2 - 0.5 * kin;                         // nuts.py:871-876
  if (isnan(energy)) energy = -INFINITY;
  const double de = energy - w.e0[c];
  const bool not_div = -de < max_energy_diff;             // nuts.py:880
  const double wsum = log_add_exp(w.sub_w[c], de);        // nuts.py:881-883
  const double thresh = de - wsum;
  const float U = draw_uniform(key, draw_site(kDrawLeafUniform, depth, leaf), (uint32_t)c);
  const bool acc = log1m_uniform(U) <= thresh;           // nuts.py:897-901
  if (acc) {
    for (int d = lane; d < D; d += 32) {
      w.sub_q[o + d] = w.end_q[side][o + d];
      w.sub_g[o + d] = Gs[o + d];
    }
  }
  if (lane == 0) {
    w.end_l[side][c] = l2;
    if (acc) { w.sub_l[c] = l2; w.sub_e[c] = energy; }
    w.sub_w[c] = wsum;
    const bool cont = not_div;                            // previous was active
    if (cont) w.sub_eds[c] += exp_nonpositive(fmin(de, 0.0));   // nuts.py:929-933
    w.sub_lf[c] += 1;                                     // nuts.py:829-830
    uint8_t nf = f;
    if (!not_div) nf &= (uint8_t)~kSubNotDiv;
    if (!(cont && no_uturn)) nf &= (uint8_t)~kSubCont;
    w.flags[c] = nf;
  }
}

__global__ void nuts_leaf_post_kernel(NutsDev w, const uint2* __restrict__ keyp, int depth,
                                      int leaf, int wslot, int r0, int r1,
                                      double max_energy_diff) {
  const int j = warp_id(), lane = threadIdx.x & 31;
  if (j >= *w.act_count) return;
  nuts_chain_leaf_post(w, w.act_idx[j], j, lane, *keyp, depth, leaf, wslot, r0, r1,
                       max_energy_diff);
}

// Tree-level biased progressive sampling and trajectory U-turn check
// (nuts.py:597-711) of a chain whose trajectory continues.
__device__ void nuts_chain_depth_end(const NutsDev& w, int c, int lane, uint2 key, int depth) {
  const uint8_t f = w.flags[c];
  const int D = vdim(w, c);
  const size_t o = voff(w, c);
  const bool sub_cont = f & kSubCont;
  const double tree_w = sub_cont ? w.sub_w[c] : -INFINITY;
  const double cw = w.cand_w[c];
  const double wsum = log_add_exp(tree_w, cw);
  double thresh = tree_w - cw;
  if (isnan(thresh)) thresh = 0.0;
  const float U = draw_uniform(key, draw_site(kDrawTreeUniform, depth, 0), (uint32_t)c);
  const bool choose = (log1m_uniform(U) <= thresh) && sub_cont;
  float dl = 0.f, dr = 0.f;   // trajectory U-turn dots, FP32 as in the reference
  for (int d = lane; d < D; d += 32) {
    if (choose) {
      w.cand_q[o + d] = w.sub_q[o + d];
      w.cand_g[o + d] = w.sub_g[o + d];
    }
    const float ms = w.mom_sum[o + d] + w.cumsum[o + d];
    w.mom_sum[o + d] = ms;
    const float im = imass(w, o, d);
    dl = fmaf(ms, w.end_p[0][o + d] * im, dl);         // momentum sum . velocities
    dr = fmaf(ms, w.end_p[1][o + d] * im, dr);
  }
  dl = warp_sum(dl);
  dr = warp_sum(dr);
  if (lane == 0) {
    if (choose) { w.cand_l[c] = w.sub_l[c]; w.cand_e[c] = w.sub_e[c]; }
    w.cand_w[c] = wsum;
    w.eds[c] += w.sub_eds[c];
    w.lf[c] += w.sub_lf[c];
    const bool no_uturn = dl >= 0.0 && dr >= 0.0;
    uint8_t nf = f;
    if (choose) nf |= kAccepted;
    if (!(sub_cont && no_uturn)) nf &= (uint8_t)~kCont;
    nf = (f & kSubNotDiv) ? (nf | kNotDiv) : (nf & (uint8_t)~kNotDiv);
    w.flags[c] = nf;
    if (nf & kCont) atomicOr(w.any_cont, 1);
  }
}

__global__ void nuts_depth_end_kernel(NutsDev w, uint2 key, int depth) {
  const int c = warp_id(), lane = threadIdx.x & 31;
  if (c >= w.C) return;
  if (!(w.flags[c] & kCont)) return;
  nuts_chain_depth_end(w, c, lane, key, depth);
}

// NUTSKernelResults of chain c (nuts.py:424-441); NULL outputs are skipped.
__device__ void nuts_chain_finalize(const NutsDev& w, int c, int lane, const NutsOutputs& out,
                                    int unrolled) {
  const size_t o = voff(w, c);
  const int D = vdim(w, c);
  for (int d = lane; d < D; d += 32) {
    if (out.state) out.state[o + d] = w.cand_q[o + d];
    if (out.grads) out.grads[o + d] = w.cand_g[o + d];
  }
  if (lane == 0) {
    const uint8_t f = w.flags[c];
    if (out.target_log_prob) out.target_log_prob[c] = w.cand_l[c];
    if (out.log_accept_ratio)
      out.log_accept_ratio[c] = log(w.eds[c] / (double)w.lf[c]);   // nuts.py:429-432
    if (out.leapfrogs_taken) out.leapfrogs_taken[c] = w.lf[c] * unrolled;
    if (out.is_accepted) out.is_accepted[c] = (f & kAccepted) ? 1 : 0;
    if (out.reach_max_depth) out.reach_max_depth[c] = (f & kCont) ? 1 : 0;
    if (out.has_divergence) out.has_divergence[c] = (f & kNotDiv) ? 0 : 1;
    if (out.energy) out.energy[c] = w.cand_e[c];
    if (out.tree_depth) out.tree_depth[c] = w.tree_depth[c];
  }
}

__global__ void nuts_finalize_kernel(NutsDev w, NutsOutputs out, int unrolled) {
  const int c = warp_id(), lane = threadIdx.x & 31;
  if (c >= w.C) return;
  nuts_chain_finalize(w, c, lane, out, unrolled);
}

// --------------------------------------------------------------------------
// Free-running NUTS: one leaf of every running chain per iteration.  The
// per-chain bodies are the lock-step kernels'; the draws are addressed by the
// chain's own transition key, depth and leaf, so a chain's transitions equal
// the lock-step sampler's with the same keys.
// --------------------------------------------------------------------------
__global__ void nuts_free_start_kernel(NutsDev w, FreeDev f, const float* __restrict__ q,
                                      const double* __restrict__ l,
                                      const float* __restrict__ g) {
  const int c = warp_id(), lane = threadIdx.x & 31;
  if (c >= w.C) return;
  const size_t o = voff(w, c);
  const int D = vdim(w, c);
  for (int d = lane; d < D; d += 32) {
    w.cand_q[o + d] = q[o + d];
    w.cand_g[o + d] = g[o + d];
  }
  if (lane == 0) {
    w.cand_l[c] = l[c];
    f.t[c] = 0;
    f.phase[c] = kPhaseStart;
    w.flags[c] = f.kmax > 0 ? kRunning : 0;
  }
}

// Start the chain's transition and/or tree depth if due, then its leaf's
// half kick + drift.
__global__ void nuts_free_prepare_kernel(NutsDev w, FreeDev f) {
  const int j = warp_id(), lane = threadIdx.x & 31;
  if (j >= *w.act_count) return;
  const int c = w.act_idx[j];
  uint8_t ph = f.phase[c];
  if (ph == kPhaseStart) {
    const uint2 key = step_key(f.seed, f.first + (uint32_t)f.t[c]);
    nuts_chain_init(w, c, lane, w.cand_q, w.cand_l, w.cand_g,
                    eps_of(f.eps_in, f.eps_per_chain, c), key);
    __syncwarp();
    if (lane == 0) {
      f.key[c] = key;
      w.flags[c] |= kRunning;
      f.depth[c] = 0;
    }
    ph = kPhaseDepth;
  }
  if (ph == kPhaseDepth) {
    __syncwarp();
    if (lane == 0) nuts_chain_depth_begin(w, c, f.key[c], f.depth[c]);
    __syncwarp();
    nuts_chain_zero_cumsum(w, c, lane);
    if (lane == 0) {
      f.leaf[c] = 0;
      f.phase[c] = kPhaseLeaf;
    }
  }
  __syncwarp();
  nuts_chain_leaf_pre(w, c, j, lane);
}

// The leaf's bookkeeping; at the end of the chain's subtree the tree-level
// step; at the end of its trajectory the transition's results go to the
// trace and the chain's next transition is due.
__global__ void nuts_free_post_kernel(NutsDev w, FreeDev f) {
  const int j = warp_id(), lane = threadIdx.x & 31;
  if (j >= *w.act_count) return;
  const int c = w.act_idx[j];
  const uint2 key = f.key[c];
  const int depth = f.depth[c], leaf = f.leaf[c];
  nuts_chain_leaf_post(w, c, j, lane, key, depth, leaf, f.wtab[leaf], f.rlo[leaf], f.rhi[leaf],
                       f.max_energy_diff);
  __syncwarp();
  if ((w.flags[c] & kSubCont) && leaf + 1 < (1 << depth)) {
    if (lane == 0) f.leaf[c] = leaf + 1;
    return;
  }
  nuts_chain_depth_end(w, c, lane, key, depth);
  __syncwarp();
  if ((w.flags[c] & kCont) && depth + 1 < f.max_depth) {
    if (lane == 0) {
      f.depth[c] = depth + 1;
      f.phase[c] = kPhaseDepth;
    }
    return;
  }
  const int t = f.t[c];
  const size_t C = (size_t)w.C;
  NutsOutputs out{f.tr_state ? f.tr_state + (size_t)t * f.tr_estride : nullptr,
                  f.tr_logp ? f.tr_logp + (size_t)t * C : nullptr, nullptr,
                  f.tr_lar ? f.tr_lar + (size_t)t * C : nullptr,
                  f.tr_lf ? f.tr_lf + (size_t)t * C : nullptr,
                  f.tr_acc ? f.tr_acc + (size_t)t * C : nullptr, nullptr,
                  f.tr_div ? f.tr_div + (size_t)t * C : nullptr, nullptr, nullptr};
  nuts_chain_finalize(w, c, lane, out, 1);
  if (f.mom_mean) {   // as moments_update_kernel, with this chain's draw count
    const size_t o = voff(w, c);
    const int D = vdim(w, c);
    const double inv_count = 1.0 / (double)(f.mom_base + t + 1);
    for (int d = lane; d < D; d += 32) {
      const double v = (double)w.cand_q[o + d];
      const double delta = v - f.mom_mean[o + d];
      const double mnew = f.mom_mean[o + d] + delta * inv_count;
      f.mom_mean[o + d] = mnew;
      f.mom_m2[o + d] += delta * (v - mnew);
    }
  }
  __syncwarp();
  if (lane == 0) {
    f.t[c] = t + 1;
    f.phase[c] = kPhaseStart;
    if (t + 1 >= f.kmax) w.flags[c] &= (uint8_t)~kRunning;
  }
}

__global__ void nuts_free_done_kernel(FreeDev f, int C, int32_t* __restrict__ out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < C) out[c] = f.t[c];
}

// --------------------------------------------------------------------------
// HMC kernels: UncalibratedHamiltonianMonteCarlo + MetropolisHastings.
// --------------------------------------------------------------------------
struct HmcDev {
  int C, D;
  float *p0, *ph, *qw, *gw;
  double* lw;
  int* count;
};

__global__ void hmc_init_kernel(HmcDev w, const float* __restrict__ q, const float* __restrict__ g,
                                const float* __restrict__ eps, int per_chain,
                                const uint2* __restrict__ keyp) {
  const uint2 key = *keyp;
  const int c = warp_id(), lane = threadIdx.x & 31;
  if (c >= w.C) return;
  if (c == 0 && lane == 0) *w.count = w.C;
  const float e = eps_of(eps, per_chain, c), he = 0.5f * e;
  const size_t o = (size_t)c * w.D;
  const uint32_t site = draw_site(kDrawMomentum, 0, 0);
  for (int d = lane; d < w.D; d += 32) {
    const float p = draw_normal(key, site, (uint32_t)(o + d));   // hmc.py:684-695
    w.p0[o + d] = p;
    const float ph = p + he * g[o + d];
    w.ph[o + d] = ph;
    w.qw[o + d] = q[o + d] + e * ph;
  }
}

__global__ void hmc_kick_drift_kernel(HmcDev w, const float* __restrict__ eps, int per_chain) {
  const int c = warp_id(), lane = threadIdx.x & 31;
  if (c >= w.C) return;
  const float e = eps_of(eps, per_chain, c);
  const size_t o = (size_t)c * w.D;
  for (int d = lane; d < w.D; d += 32) {
    const float ph = w.ph[o + d] + e * w.gw[o + d];
    w.ph[o + d] = ph;
    w.qw[o + d] = w.qw[o + d] + e * ph;
  }
}

__global__ void hmc_finish_kernel(HmcDev w, const float* __restrict__ q0,
                                  const double* __restrict__ l0, const float* __restrict__ g0,
                                  const float* __restrict__ eps, int per_chain,
                                  const uint2* __restrict__ keyp,
                                  HmcOutputs out) {
  const uint2 key = *keyp;
  const int c = warp_id(), lane = threadIdx.x & 31;
  if (c >= w.C) return;
  const float e = eps_of(eps, per_chain, c), he = 0.5f * e;
  const size_t o = (size_t)c * w.D;
  float k0l = 0.f, k1l = 0.f;   // per-lane FP32 shares of |p|^2, summed in FP64
  for (int d = lane; d < w.D; d += 32) {
    const float g = w.gw[o + d];
    const float p1 = (w.ph[o + d] + e * g) - he * g;
    const float p0 = w.p0[o + d];
    k0l = fmaf(p0, p0, k0l);
    k1l = fmaf(p1, p1, k1l);
    if (out.final_momentum) out.final_momentum[o + d] = p1;
    if (out.initial_momentum) out.initial_momentum[o + d] = p0;
    if (out.proposed_state) out.proposed_state[o + d] = w.qw[o + d];
    if (out.proposed_grads) out.proposed_grads[o + d] = g;
  }
  const double k0 = warp_sum((double)k0l);
  const double k1 = warp_sum((double)k1l);
  const double l1 = w.lw[c];
  double corr = k0 - k1;                                  // hmc.py:861-875
  corr = isfinite(corr) ? 0.5 * corr : -INFINITY;
  double lar = l1 - l0[c] + corr;                         // metropolis_hastings.py:204-215
  if (!isfinite(lar)) lar = -INFINITY;
  const float U = draw_uniform(key, draw_site(kDrawMhUniform, 0, 0), (uint32_t)c);
  const bool acc = log((double)U) < lar;                  // metropolis_hastings.py:221-227
  for (int d = lane; d < w.D; d += 32) {
    out.next_state[o + d] = acc ? w.qw[o + d] : q0[o + d];
    out.next_grads[o + d] = acc ? w.gw[o + d] : g0[o + d];
  }
  if (lane == 0) {
    out.next_tlp[c] = acc ? l1 : l0[c];
    if (out.proposed_tlp) out.proposed_tlp[c] = l1;
    if (out.log_acceptance_correction) out.log_acceptance_correction[c] = corr;
    out.log_accept_ratio[c] = lar;
    out.is_accepted[c] = acc ? 1 : 0;
  }
}

// MetropolisHastings.one_step's correction for a proposal another kernel made
// (metropolis_hastings.py:160-254): log_accept_ratio = safe_sum(proposed -
// current + correction) (non-finite -> -inf), accept iff log U < ratio with
// U the transition's MH uniform (the draw hmc_finish_kernel uses, so
// MetropolisHastings(UncalibratedHamiltonianMonteCarlo) reproduces
// HamiltonianMonteCarlo bit for bit), next = accepted ? proposed : current.
__global__ void mh_accept_kernel(int C, int D, uint2 key, const double* __restrict__ cur_tlp,
                                 const double* __restrict__ prop_tlp,
                                 const double* __restrict__ corr,
                                 const float* __restrict__ cur_q, const float* __restrict__ prop_q,
                                 float* __restrict__ next_q, double* __restrict__ lar_out,
                                 uint8_t* __restrict__ acc_out) {
  const int c = warp_id(), lane = threadIdx.x & 31;
  if (c >= C) return;
  double lar = prop_tlp[c] - cur_tlp[c] + (corr ? corr[c] : 0.0);
  if (!isfinite(lar)) lar = -INFINITY;
  const float U = draw_uniform(key, draw_site(kDrawMhUniform, 0, 0), (uint32_t)c);
  const bool acc = log((double)U) < lar;
  const size_t o = (size_t)c * D;
  for (int d = lane; d < D; d += 32) next_q[o + d] = acc ? prop_q[o + d] : cur_q[o + d];
  if (lane == 0) {
    lar_out[c] = lar;
    acc_out[c] = acc ? 1 : 0;
  }
}

void metropolis_hastings_step(cudaStream_t s, int64_t C, int64_t D, uint2 key,
                              const double* cur_tlp, const double* prop_tlp, const double* corr,
                              const float* cur_q, const float* prop_q, float* next_q,
                              double* lar, uint8_t* acc) {
  mh_accept_kernel<<<warp_blocks(C), 32 * kWarpsPerBlock, 0, s>>>(
      (int)C, (int)D, key, cur_tlp, prop_tlp, corr, cur_q, prop_q, next_q, lar, acc);
  GBM_CUDA(cudaGetLastError());
}

// --------------------------------------------------------------------------
// Dual averaging (dual_averaging_step_size_adaptation.py:353-475)
// --------------------------------------------------------------------------
// state: [groups][4] doubles = error_sum, log_averaging_step, log_shrinkage_target, step.
// `reduced` (optional, float64 [groups]): the caller's reduction of the log
// accept probabilities (a custom reduce_fn, :141,410-422); `lar` is then
// unused.
__global__ void dual_averaging_kernel(const double* __restrict__ lar, int C, int per_chain,
                                      DaParams prm, const double* __restrict__ target_accept,
                                      double* __restrict__ state, float* __restrict__ eps,
                                      const double* __restrict__ reduced, int groups) {
  __shared__ double red[32];
  __shared__ double bcast;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int nw = (blockDim.x + 31) >> 5;
  auto lap = [&](int c) {  // simple_step_size_adaptation.py:42-48
    double v = lar[c];
    if (!isfinite(v)) v = -INFINITY;
    return fmin(v, 0.0);
  };
  auto update = [&](int g, double reduced) {
    double* st = state + 4 * g;
    const double tgt = target_accept ? target_accept[g] : prm.target_accept_prob;
    const double err = st[0] + tgt - exp(reduced);
    const double step = st[3] + 1.0;
    const double soft_t = prm.step_count_smoothing + step;
    const double new_log_step = st[2] - (err * sqrt(step)) / (soft_t * prm.exploration_shrinkage);
    const double eta = pow(step, -prm.decay_rate);
    double new_log_avg = eta * new_log_step + (1.0 - eta) * st[1];
    const int istep = (int)step;
    const float cur = eps[g];
    float ns;
    if (istep < prm.num_adaptation_steps) ns = (float)exp(new_log_step);
    else if (istep > prm.num_adaptation_steps) ns = cur;
    else ns = (float)exp(new_log_avg);
    if (istep > prm.num_adaptation_steps) new_log_avg = st[1];
    st[0] = err;
    st[1] = new_log_avg;
    st[3] = step;
    eps[g] = ns;
  };
  if (reduced) {
    for (int g = tid; g < groups; g += blockDim.x) update(g, reduced[g]);
    return;
  }
  if (per_chain) {
    for (int c = tid; c < C; c += blockDim.x) update(c, lap(c));
    return;
  }
  // reduce_logmeanexp over all chains (math/generic.py:221-275).
  double m = -INFINITY;
  for (int c = tid; c < C; c += blockDim.x) m = fmax(m, lap(c));
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if (lane == 0) red[wid] = m;
  __syncthreads();
  if (tid == 0) {
    double mm = -INFINITY;
    for (int i = 0; i < nw; ++i) mm = fmax(mm, red[i]);
    bcast = isfinite(mm) ? mm : 0.0;
  }
  __syncthreads();
  const double mx = bcast;
  double s = 0.0;
  for (int c = tid; c < C; c += blockDim.x) s += exp(lap(c) - mx);
  s = warp_sum(s);
  __syncthreads();
  if (lane == 0) red[wid] = s;
  __syncthreads();
  if (tid == 0) {
    double tot = 0.0;
    for (int i = 0; i < nw; ++i) tot += red[i];
    update(0, log(tot) + mx - log((double)C));
  }
}

// --------------------------------------------------------------------------
// Host orchestration
// --------------------------------------------------------------------------

// nuts.py:1013-1071, restated: the slot each leaf writes (-1: nothing to
// keep) and the slot range [lo, hi) it checks for a U-turn.
void nuts_instructions(int depth, std::vector<int>* write, std::vector<int>* lo,
                       std::vector<int>* hi, int* slots) {
  const int n = 1 << depth;
  std::vector<int> last_end(n, -1);
  std::vector<std::vector<int>> ends_at(n);
  for (int h = 1; h <= depth; ++h) {
    const int size = 1 << h;
    for (int a = 0; a < n; a += size) {
      last_end[a] = std::max(last_end[a], a + size - 1);
      ends_at[a + size - 1].push_back(a);
    }
  }
  write->assign(n, -1);
  lo->assign(n, 0);
  hi->assign(n, 0);
  int max_slot = 0;
  for (int j = 0; j < n; ++j) {
    std::vector<int> alive;
    for (int i = 0; i <= j; ++i)
      if (last_end[i] >= j) alive.push_back(i);
    if (last_end[j] >= 0) {
      (*write)[j] = (int)alive.size() - 1;
      max_slot = std::max(max_slot, (*write)[j]);
    }
    if (!ends_at[j].empty()) {
      const int first = *std::min_element(ends_at[j].begin(), ends_at[j].end());
      const int r0 = (int)(std::find(alive.begin(), alive.end(), first) - alive.begin());
      (*lo)[j] = r0;
      (*hi)[j] = r0 + (int)ends_at[j].size();
    }
  }
  *slots = max_slot + 1;
}

void nuts_setup(gbm_nuts* k) {
  int slots = 0;
  nuts_instructions(k->max_tree_depth, &k->write_instr, &k->read_lo, &k->read_hi, &slots);
  const Target* t = k->target->impl.get();
  const int64_t C = k->max_chains, D = t->dim;
  NutsDev& w = k->dev;
  w.C = (int)C;
  w.D = (int)D;
  w.slots = slots;
  w.ragged = t->ragged_offsets() != nullptr;
  w.coff = t->ragged_offsets();
  w.cdim = t->ragged_dims();
  // Carve one allocation: float vectors, slot memory, doubles, ints, bytes.
  const size_t vec = w.ragged ? (size_t)t->ragged_elements() : (size_t)C * D;
  const size_t n_float_vecs = 6 + 6 + 2;   // ends(6), cand/sub/mom/cumsum(6), qw/gw(2)
  size_t bytes = 0;
  auto take = [&](size_t b) { size_t at = bytes; bytes += (b + 255) / 256 * 256; return at; };
  size_t off_f = take(sizeof(float) * vec * n_float_vecs);
  size_t off_slots = take(sizeof(float) * vec * slots * 2);
  size_t off_d = take(sizeof(double) * C * 12);
  const size_t nblk = (size_t)((C + 1023) / 1024);
  size_t off_i = take(sizeof(int) * (C * 4 + 16 + nblk));
  size_t off_b = take(C);
  size_t off_e = take(sizeof(float) * C);
  k->mem.reserve(bytes);
  char* base = k->mem.as<char>();
  float* fv = reinterpret_cast<float*>(base + off_f);
  w.end_q[0] = fv + 0 * vec; w.end_q[1] = fv + 1 * vec;
  w.end_p[0] = fv + 2 * vec; w.end_p[1] = fv + 3 * vec;
  w.end_g[0] = fv + 4 * vec; w.end_g[1] = fv + 5 * vec;
  w.cand_q = fv + 6 * vec; w.cand_g = fv + 7 * vec;
  w.sub_q = fv + 8 * vec; w.sub_g = fv + 9 * vec;
  w.mom_sum = fv + 10 * vec; w.cumsum = fv + 11 * vec;
  w.qw = fv + 12 * vec; w.gw = fv + 13 * vec;
  float* sv = reinterpret_cast<float*>(base + off_slots);
  w.slot_p = sv;
  w.slot_cs = sv + vec * slots;
  double* dv = reinterpret_cast<double*>(base + off_d);
  w.end_l[0] = dv + 0 * C; w.end_l[1] = dv + 1 * C;
  w.cand_l = dv + 2 * C; w.cand_e = dv + 3 * C; w.cand_w = dv + 4 * C;
  w.sub_l = dv + 5 * C; w.sub_e = dv + 6 * C; w.sub_w = dv + 7 * C;
  w.e0 = dv + 8 * C; w.eds = dv + 9 * C; w.sub_eds = dv + 10 * C; w.lw = dv + 11 * C;
  int* iv = reinterpret_cast<int*>(base + off_i);
  w.lf = iv; w.sub_lf = iv + C; w.tree_depth = iv + 2 * C; w.act_idx = iv + 3 * C;
  w.act_count = iv + 4 * C; w.any_cont = iv + 4 * C + 1; w.act_blk = iv + 4 * C + 16;
  w.flags = reinterpret_cast<uint8_t*>(base + off_b);
  w.eps = reinterpret_cast<float*>(base + off_e);
  GBM_CUDA(cudaMemsetAsync(base, 0, bytes, k->ctx->stream));
  k->target_ws.reserve(k->target->impl->workspace_bytes(C));
  for (auto& ev : k->poll_events) GBM_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  k->key_dev.reserve(sizeof(uint2));
  // Batches of leaves are captured on a private stream (the caller's may be
  // the legacy default stream, which cannot be captured) and the executable
  // graphs are launched on the caller's stream.
  GBM_CUDA(cudaStreamCreateWithFlags(&k->graph_stream, cudaStreamNonBlocking));
  k->use_graphs = true;
}

void nuts_clear_graphs(gbm_nuts* k) {
  for (auto& g : k->graphs) cudaGraphExecDestroy(g.second);
  k->graphs.clear();
}

void nuts_release_graphs(gbm_nuts* k) {
  for (auto& g : k->graphs) cudaGraphExecDestroy(g.second);
  k->graphs.clear();
  if (k->graph_stream) cudaStreamDestroy(k->graph_stream);
  k->graph_stream = nullptr;
}

static void nuts_eval(gbm_nuts* k, cudaStream_t s, bool capturing = false) {
  const NutsDev& w = k->dev;
  if (k->profiling && !capturing) {
    if (k->prof_used + 2 > k->prof_events.size()) {
      cudaEvent_t a, b;
      GBM_CUDA(cudaEventCreate(&a));
      GBM_CUDA(cudaEventCreate(&b));
      k->prof_events.push_back(a);
      k->prof_events.push_back(b);
    }
    GBM_CUDA(cudaEventRecord(k->prof_events[k->prof_used], s));
  }
  if (w.ragged)
    k->target->impl->eval_active(w.qw, w.act_idx, w.act_count, w.lw, w.gw, k->target_ws.ptr, s);
  else
    k->target->impl->eval(w.qw, w.D, w.act_count, w.C, w.lw, w.gw, w.D, k->target_ws.ptr, s);
  if (!capturing) k->prof_launches += k->target->impl->launches_per_eval(w.C);
  if (k->profiling && !capturing) {
    GBM_CUDA(cudaEventRecord(k->prof_events[k->prof_used + 1], s));
    k->prof_used += 2;
    ++k->prof_evals;
  }
}

// Sum the recorded (start, end) pairs; the stream must be synchronized.
void nuts_profile_flush(gbm_nuts* k) {
  for (size_t i = 0; i + 1 < k->prof_used; i += 2) {
    float ms = 0.f;
    GBM_CUDA(cudaEventElapsedTime(&ms, k->prof_events[i], k->prof_events[i + 1]));
    k->prof_eval_ms += ms;
  }
  k->prof_used = 0;
}

void nuts_one_step(gbm_nuts* k, int64_t chains, const float* q, const double* l, const float* g,
                   const float* eps, int eps_per_chain, uint2 key, const NutsOutputs& out) {
  gbm_context* ctx = k->target->ctx;
  cudaStream_t s = ctx->stream;
  NutsDev w = k->dev;
  w.C = (int)chains;
  w.inv_mass = k->inv_mass;
  w.im_per_chain = k->im_per_chain;
  int* host_flags = ctx->host_flags;
  const int wb = warp_blocks(chains), tb = 256;
  const uint2* keyp = k->key_dev.as<uint2>();
  set_key_kernel<<<1, 1, 0, s>>>(k->key_dev.as<uint2>(), key);
  nuts_init_kernel<<<wb, 32 * kWarpsPerBlock, 0, s>>>(w, q, l, g, eps, eps_per_chain, key);
  GBM_CUDA(cudaGetLastError());
  k->last_leaf_iterations = 0;
  // One leaf: half kick + drift, gradient, final kick and tree bookkeeping,
  // then the next active list (on stream ls: the caller's, or the capture
  // stream while a graph is recorded).
  auto leaf_step = [&](int depth, int leaf, bool capturing, cudaStream_t ls) {
    nuts_leaf_pre_kernel<<<wb, 32 * kWarpsPerBlock, 0, ls>>>(w);
    nuts_eval(k, ls, capturing);
    for (int u = 1; u < k->unrolled_leapfrog_steps; ++u) {
      nuts_leaf_mid_kernel<<<wb, 32 * kWarpsPerBlock, 0, ls>>>(w);
      nuts_eval(k, ls, capturing);
    }
    nuts_leaf_post_kernel<<<wb, 32 * kWarpsPerBlock, 0, ls>>>(
        w, keyp, depth, leaf, k->write_instr[leaf], k->read_lo[leaf], k->read_hi[leaf],
        k->max_energy_diff);
    GBM_CUDA(cudaGetLastError());
    build_active(w, kSubCont, ls);
    if (!capturing)
      k->prof_launches += 2 + active_launches(w.C) + (k->unrolled_leapfrog_steps - 1);
  };
  // Profiled steps time every gradient evaluation with events: leaf by leaf.
  const bool graphs = k->use_graphs && !k->profiling;
  for (int depth = 0; depth < k->max_tree_depth; ++depth) {
    if (depth > 0) {
      GBM_CUDA(cudaMemcpyAsync(host_flags, w.any_cont, sizeof(int), cudaMemcpyDeviceToHost, s));
      GBM_CUDA(cudaStreamSynchronize(s));
      if (k->profiling) nuts_profile_flush(k);
      check_device_error(ctx);
      if (host_flags[0] == 0) break;
    }
    nuts_depth_begin_kernel<<<(int)((chains + tb - 1) / tb), tb, 0, s>>>(w, key, depth);
    nuts_zero_cumsum_kernel<<<wb, 32 * kWarpsPerBlock, 0, s>>>(w);
    build_active(w, kSubCont, s);
    const int leaves = 1 << depth;
    const int batch = 8;
    for (int leaf = 0; leaf < leaves; ++leaf) {
      // Stop launching once every chain's subtree has terminated: poll the
      // active count recorded at the previous batch boundary (the host runs
      // at most one batch of leaves ahead of the device).
      if (leaf % batch == 0 && leaf > 0) {
        const int b = leaf / batch;
        const int slot = b % 4;
        GBM_CUDA(cudaMemcpyAsync(host_flags + 1 + slot, w.act_count, sizeof(int),
                                 cudaMemcpyDeviceToHost, s));
        GBM_CUDA(cudaEventRecord(k->poll_events[slot], s));
        if (b >= 2) {
          const int prev = (b - 1) % 4;
          GBM_CUDA(cudaEventSynchronize(k->poll_events[prev]));
          if (host_flags[1 + prev] == 0) break;
        }
      }
      if (graphs && leaf % batch == 0) {
        // The next `nl` leaves as one graph launch (leaves whose subtree has
        // ended cost a launch of idle warps only).
        const int nl = std::min(batch, leaves - leaf);
        const int64_t gkey = ((int64_t)chains << 32) | ((int64_t)depth << 16) | leaf;
        auto it = k->graphs.find(gkey);
        if (it == k->graphs.end()) {
          cudaGraph_t graph;
          cudaStream_t cs = k->graph_stream;
          GBM_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
          for (int l = leaf; l < leaf + nl; ++l) leaf_step(depth, l, true, cs);
          GBM_CUDA(cudaStreamEndCapture(cs, &graph));
          cudaGraphExec_t exec;
          GBM_CUDA(cudaGraphInstantiate(&exec, graph, 0));
          GBM_CUDA(cudaGraphDestroy(graph));
          it = k->graphs.emplace(gkey, exec).first;
        }
        GBM_CUDA(cudaGraphLaunch(it->second, s));
        ++k->graph_launches;
        k->prof_launches += (int64_t)nl * (2 + active_launches(w.C) +
                                           k->unrolled_leapfrog_steps * (
            k->target->impl->launches_per_eval(chains) + 1) - 1);
        k->last_leaf_iterations += nl;
        leaf += nl - 1;
        continue;
      }
      leaf_step(depth, leaf, false, s);
      ++k->last_leaf_iterations;
    }
    nuts_depth_end_kernel<<<wb, 32 * kWarpsPerBlock, 0, s>>>(w, key, depth);
    GBM_CUDA(cudaGetLastError());
    k->prof_launches += 3 + active_launches(w.C);
  }
  nuts_finalize_kernel<<<wb, 32 * kWarpsPerBlock, 0, s>>>(w, out, k->unrolled_leapfrog_steps);
  GBM_CUDA(cudaGetLastError());
  k->prof_launches += 2;
}

int64_t nuts_run_free(gbm_nuts* k, int64_t chains, const float* q, const double* l,
                      const float* g, const float* eps, int eps_per_chain, uint2 seed,
                      uint32_t first_step, int kmax, int64_t max_leaf_iterations, FreeDev f,
                      int32_t* transitions_done) {
  gbm_context* ctx = k->target->ctx;
  cudaStream_t s = ctx->stream;
  NutsDev w = k->dev;
  w.C = (int)chains;
  w.inv_mass = k->inv_mass;
  w.im_per_chain = k->im_per_chain;
  const int C = (int)chains;
  const int leaves = 1 << k->max_tree_depth;
  // Per-chain loop state and the leaf tables (device), carved from free_mem.
  const size_t tab = ((size_t)leaves * 3 * sizeof(int) + 255) / 256 * 256;
  const size_t per = ((size_t)C * (3 * sizeof(int) + sizeof(uint2) + 1) + 255) / 256 * 256;
  if (k->free_mem.bytes < tab + per) {
    GBM_CUDA(cudaStreamSynchronize(s));
    k->free_mem.reserve(tab + per);
  }
  char* base = k->free_mem.as<char>();
  int* tabs = reinterpret_cast<int*>(base);
  std::vector<int> host_tab(3 * leaves);
  std::copy(k->write_instr.begin(), k->write_instr.end(), host_tab.begin());
  std::copy(k->read_lo.begin(), k->read_lo.end(), host_tab.begin() + leaves);
  std::copy(k->read_hi.begin(), k->read_hi.end(), host_tab.begin() + 2 * leaves);
  GBM_CUDA(cudaMemcpyAsync(tabs, host_tab.data(), sizeof(int) * 3 * leaves,
                           cudaMemcpyHostToDevice, s));
  GBM_CUDA(cudaStreamSynchronize(s));   // host_tab is freed on return
  f.wtab = tabs;
  f.rlo = tabs + leaves;
  f.rhi = tabs + 2 * leaves;
  char* pc = base + tab;
  f.key = reinterpret_cast<uint2*>(pc);
  f.t = reinterpret_cast<int*>(pc + sizeof(uint2) * C);
  f.depth = f.t + C;
  f.leaf = f.t + 2 * C;
  f.phase = reinterpret_cast<uint8_t*>(f.t + 3 * C);
  f.eps_in = eps;
  f.eps_per_chain = eps_per_chain;
  f.seed = seed;
  f.first = first_step;
  f.kmax = kmax;
  f.max_depth = k->max_tree_depth;
  f.max_energy_diff = k->max_energy_diff;
  const int wb = warp_blocks(chains);
  nuts_free_start_kernel<<<wb, 32 * kWarpsPerBlock, 0, s>>>(w, f, q, l, g);
  GBM_CUDA(cudaGetLastError());
  k->prof_launches += 1;
  auto iteration = [&](cudaStream_t ls, bool capturing) {
    build_active(w, kRunning, ls);
    nuts_free_prepare_kernel<<<wb, 32 * kWarpsPerBlock, 0, ls>>>(w, f);
    nuts_eval(k, ls, capturing);
    nuts_free_post_kernel<<<wb, 32 * kWarpsPerBlock, 0, ls>>>(w, f);
    GBM_CUDA(cudaGetLastError());
    if (!capturing) k->prof_launches += 2 + active_launches(C);
  };
  // Batches of `batch` iterations, replayed as one CUDA graph (captured for
  // this call: its pointers are the call's); the host polls the running count
  // recorded after each batch, at most two batches behind the device.
  const int batch = 8;
  cudaGraphExec_t exec = nullptr;
  const bool graphs = k->use_graphs && !k->profiling;
  if (graphs) {
    cudaGraph_t graph;
    cudaStream_t cs = k->graph_stream;
    GBM_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    for (int i = 0; i < batch; ++i) iteration(cs, true);
    GBM_CUDA(cudaStreamEndCapture(cs, &graph));
    GBM_CUDA(cudaGraphInstantiate(&exec, graph, 0));
    GBM_CUDA(cudaGraphDestroy(graph));
  }
  int* host_flags = ctx->host_flags;
  int64_t iters = 0;
  int64_t b = 0;
  try {
    while (iters < max_leaf_iterations) {
      const int64_t n = std::min<int64_t>(batch, max_leaf_iterations - iters);
      if (exec && n == batch) {
        GBM_CUDA(cudaGraphLaunch(exec, s));
        k->prof_launches +=
            (int64_t)batch * (2 + active_launches(C) + k->target->impl->launches_per_eval(C));
      } else {
        for (int64_t i = 0; i < n; ++i) iteration(s, false);
      }
      iters += n;
      const int slot = (int)(b % 4);
      GBM_CUDA(cudaMemcpyAsync(host_flags + 1 + slot, w.act_count, sizeof(int),
                               cudaMemcpyDeviceToHost, s));
      GBM_CUDA(cudaEventRecord(k->poll_events[slot], s));
      if (b >= 1) {
        const int prev = (int)((b - 1) % 4);
        GBM_CUDA(cudaEventSynchronize(k->poll_events[prev]));
        check_device_error(ctx);
        // The running count of two batches ago bounds the work left: stop
        // once no chain was running then.
        if (host_flags[1 + prev] == 0) break;
      }
      ++b;
    }
  } catch (...) {
    if (exec) cudaGraphExecDestroy(exec);
    throw;
  }
  if (exec) {
    GBM_CUDA(cudaStreamSynchronize(s));
    GBM_CUDA(cudaGraphExecDestroy(exec));
  }
  if (transitions_done) {
    nuts_free_done_kernel<<<(C + 255) / 256, 256, 0, s>>>(f, C, transitions_done);
    GBM_CUDA(cudaGetLastError());
  }
  k->last_leaf_iterations = iters;
  return iters;
}

void hmc_setup(gbm_hmc* k) {
  const int64_t C = k->max_chains, D = k->target->impl->dim;
  const size_t vec = (size_t)C * D;
  k->mem.reserve(sizeof(float) * vec * 4 + sizeof(double) * C + 256 + sizeof(int) * 64);
  k->target_ws.reserve(k->target->impl->workspace_bytes(C));
  k->key_dev.reserve(16);
}

void hmc_one_step(gbm_hmc* k, int64_t chains, const float* q, const double* l, const float* g,
                  const float* eps, int per_chain, int num_leapfrog_steps, uint2 key,
                  const HmcOutputs& out) {
  cudaStream_t s = k->target->ctx->stream;
  uint2* keyp = k->key_dev.as<uint2>();
  set_key_kernel<<<1, 1, 0, s>>>(keyp, key);
  hmc_step_launches(k, chains, q, l, g, eps, per_chain, num_leapfrog_steps, keyp, out, s);
}

void hmc_step_launches(gbm_hmc* k, int64_t chains, const float* q, const double* l,
                       const float* g, const float* eps, int per_chain, int num_leapfrog_steps,
                       const uint2* keyp, const HmcOutputs& out, cudaStream_t s) {
  const int64_t D = k->target->impl->dim;
  const size_t vec = (size_t)k->max_chains * D;
  float* fv = k->mem.as<float>();
  HmcDev w;
  w.C = (int)chains;
  w.D = (int)D;
  w.p0 = fv;
  w.ph = fv + vec;
  w.qw = fv + 2 * vec;
  w.gw = fv + 3 * vec;
  w.lw = reinterpret_cast<double*>(fv + 4 * vec);
  w.count = reinterpret_cast<int*>(w.lw + k->max_chains);
  const int wb = warp_blocks(chains);
  hmc_init_kernel<<<wb, 32 * kWarpsPerBlock, 0, s>>>(w, q, g, eps, per_chain, keyp);
  GBM_CUDA(cudaGetLastError());
  for (int i = 0; i < num_leapfrog_steps; ++i) {
    k->target->impl->eval(w.qw, w.D, w.count, w.C, w.lw, w.gw, w.D, k->target_ws.ptr, s);
    if (i + 1 < num_leapfrog_steps)
      hmc_kick_drift_kernel<<<wb, 32 * kWarpsPerBlock, 0, s>>>(w, eps, per_chain);
  }
  hmc_finish_kernel<<<wb, 32 * kWarpsPerBlock, 0, s>>>(w, q, l, g, eps, per_chain, keyp, out);
  GBM_CUDA(cudaGetLastError());
}

void dual_averaging_update(cudaStream_t s, const double* lar, int64_t C, int per_chain,
                           const DaParams& prm, const double* target_accept, double* state,
                           float* eps) {
  dual_averaging_kernel<<<1, 1024, 0, s>>>(lar, (int)C, per_chain, prm, target_accept, state, eps,
                                           nullptr, 0);
  GBM_CUDA(cudaGetLastError());
}

void dual_averaging_update_reduced(cudaStream_t s, const double* reduced, int64_t groups,
                                   const DaParams& prm, const double* target_accept,
                                   double* state, float* eps) {
  dual_averaging_kernel<<<1, 1024, 0, s>>>(nullptr, 0, 0, prm, target_accept, state, eps,
                                           reduced, (int)groups);
  GBM_CUDA(cudaGetLastError());
}

}  // namespace gbm
