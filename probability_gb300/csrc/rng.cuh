// Counter-based draws for the samplers: Philox4x32-10 (Salmon et al., SC'11).
//
// Addressing (mirrored by the CPU oracle's philox module):
//   key     = 2 x uint32 per-transition seed
//   counter = (element, (kind << 24) | (depth << 16) | leaf, 0, 0)
// element = chain * dim + d for momentum, chain for per-chain scalars.
// A draw therefore depends only on (key, kind, depth, leaf, element): the
// engine may skip or compact finished chains without changing any other
// chain's draws.
#pragma once
#include <stdint.h>

namespace gbm {

enum DrawKind : uint32_t {
  kDrawMomentum = 1,
  kDrawDirection = 2,
  kDrawLeafUniform = 3,
  kDrawTreeUniform = 4,
  kDrawMhUniform = 5,
  kDrawStepKey = 6,
};

__host__ __device__ __forceinline__ uint32_t mulhi32(uint32_t a, uint32_t b) {
#ifdef __CUDA_ARCH__
  return __umulhi(a, b);
#else
  return (uint32_t)(((uint64_t)a * (uint64_t)b) >> 32);
#endif
}

__host__ __device__ __forceinline__ uint4 philox4x32_10(uint2 key, uint4 c) {
#pragma unroll
  for (int i = 0; i < 10; ++i) {
    const uint32_t hi0 = mulhi32(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
    const uint32_t hi1 = mulhi32(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
    c = make_uint4(hi1 ^ c.y ^ key.x, lo1, hi0 ^ c.w ^ key.y, lo0);
    key.x += 0x9E3779B9u;
    key.y += 0xBB67AE85u;
  }
  return c;
}

__host__ __device__ __forceinline__ uint32_t draw_site(uint32_t kind, uint32_t depth,
                                                       uint32_t leaf) {
  return (kind << 24) | (depth << 16) | leaf;
}

__device__ __forceinline__ uint4 draw_bits(uint2 key, uint32_t site, uint32_t elem) {
  return philox4x32_10(key, make_uint4(elem, site, 0u, 0u));
}

// Uniform in [0, 1) with 24 random bits (exact in float32).
__device__ __forceinline__ float draw_uniform(uint2 key, uint32_t site, uint32_t elem) {
  return (float)(draw_bits(key, site, elem).x >> 8) * 0x1p-24f;
}

// Box-Muller normal from the first two words: sqrt(-2 log u1) cos(2 pi u2),
// u1 in (0, 1], u2 in [0, 1).
__device__ __forceinline__ float draw_normal(uint2 key, uint32_t site, uint32_t elem) {
  const uint4 o = draw_bits(key, site, elem);
  const float u1 = (float)((o.x >> 8) + 1u) * 0x1p-24f;
  const float u2 = (float)(o.y >> 8) * 0x1p-24f;
  return sqrtf(-2.f * logf(u1)) * cospif(2.f * u2);
}

__device__ __forceinline__ int draw_direction(uint2 key, uint32_t depth, uint32_t chain) {
  return (int)(draw_bits(key, draw_site(kDrawDirection, depth, 0), chain).x >> 31);
}

// Per-transition key of the device-side chain loop: Philox(seed; step).
__host__ __device__ __forceinline__ uint2 step_key(uint2 seed, uint32_t step) {
  const uint4 o = philox4x32_10(seed, make_uint4(step, draw_site(kDrawStepKey, 0, 0), 0u, 0u));
  return make_uint2(o.x, o.y);
}

}  // namespace gbm
