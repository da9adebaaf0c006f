"""NumPy mirror of the engine's Philox4x32-10 draw stream (oracle side).

Philox4x32-10 is the counter-based generator of Salmon, Moraes, Dror and Shaw,
"Parallel random numbers: as easy as 1, 2, 3" (SC'11).  The round function,
multipliers and Weyl key increments below are the published ones; the
known-answer vectors in ``tests/golden/philox_kat.json`` pin them.

Draw addressing (shared with ``probability_gb300/csrc/rng.cuh``):

  key     = the 2 x uint32 per-transition seed
  counter = (element, (kind << 24) | (depth << 16) | leaf, hi, 0)

``element`` is ``chain * dim + d`` for momentum and ``chain`` for per-chain
scalars.  ``kind`` codes are listed in ``KIND``.  This replaces the
reference's ``samplers.split_seed``/``samplers.normal``/``samplers.uniform``
(internal/samplers.py:217,308,356) with an addressable stream: a draw's value
does not depend on how many other chains are still active, which is what lets
the engine compact finished chains without changing any chain's result.
"""
import numpy as np

MASK32 = np.uint64(0xFFFFFFFF)
M0 = np.uint64(0xD2511F53)
M1 = np.uint64(0xCD9E8D57)
W0 = np.uint64(0x9E3779B9)
W1 = np.uint64(0xBB67AE85)

KIND = dict(momentum=1, direction=2, leaf_uniform=3, tree_uniform=4,
            mh_uniform=5, step_key=6)


def philox4x32_10(key, ctr):
  """Philox4x32 with 10 rounds.  key: (k0, k1); ctr: 4 arrays of uint32."""
  k0 = np.uint64(int(key[0]) & 0xFFFFFFFF)
  k1 = np.uint64(int(key[1]) & 0xFFFFFFFF)
  c0, c1, c2, c3 = [np.asarray(c, dtype=np.uint64) & MASK32 for c in ctr]
  for _ in range(10):
    p0 = M0 * c0
    p1 = M1 * c2
    hi0, lo0 = p0 >> np.uint64(32), p0 & MASK32
    hi1, lo1 = p1 >> np.uint64(32), p1 & MASK32
    c0, c1, c2, c3 = (hi1 ^ c1 ^ k0) & MASK32, lo1, (hi0 ^ c3 ^ k1) & MASK32, lo0
    k0 = (k0 + W0) & MASK32
    k1 = (k1 + W1) & MASK32
  return (c0.astype(np.uint32), c1.astype(np.uint32),
          c2.astype(np.uint32), c3.astype(np.uint32))


def _site(kind, depth=0, leaf=0):
  return np.uint64((KIND[kind] << 24) | (int(depth) << 16) | int(leaf))


def _bits(key, kind, n, depth=0, leaf=0):
  elem = np.arange(n, dtype=np.uint64)
  z = np.zeros_like(elem)
  return philox4x32_10(key, (elem, z + _site(kind, depth, leaf), z, z))


def uniform(key, kind, n, depth=0, leaf=0):
  """float32 uniforms in [0, 1): 24 high bits of the first output word."""
  o0, _, _, _ = _bits(key, kind, n, depth, leaf)
  return ((o0 >> np.uint32(8)).astype(np.float64) * 2.0 ** -24).astype(np.float32)


def normal(key, kind, shape, depth=0, leaf=0):
  """Box-Muller normals from the first two output words (one per element).

  u1 = (hi24(o0) + 1) / 2^24 in (0, 1], u2 = hi24(o1) / 2^24 in [0, 1),
  z = sqrt(-2 log u1) * cos(2 pi u2).  Evaluated in float64 and rounded to
  float32; the engine evaluates it in float32, so the two agree to a few ulp.
  """
  n = int(np.prod(shape))
  o0, o1, _, _ = _bits(key, kind, n, depth, leaf)
  u1 = ((o0 >> np.uint32(8)).astype(np.float64) + 1.0) * 2.0 ** -24
  u2 = (o1 >> np.uint32(8)).astype(np.float64) * 2.0 ** -24
  z = np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)
  return z.astype(np.float32).reshape(shape)


def direction(key, n, depth):
  """Per-chain tree-doubling direction in {0, 1} (1 = forward)."""
  o0, _, _, _ = _bits(key, 'direction', n, depth, 0)
  return (o0 >> np.uint32(31)).astype(np.int32)


def step_key(seed, step):
  """Per-transition key of ``sample_chain``: Philox(seed; step, STEP_KEY)."""
  o0, o1, _, _ = philox4x32_10(
      seed, (np.array([step], np.uint64), np.array([_site('step_key')]),
             np.zeros(1, np.uint64), np.zeros(1, np.uint64)))
  return (int(o0[0]), int(o1[0]))


class PhiloxDraws:
  """Draw source for one transition, in the order the reference consumes them.

  HMC (hmc.py:684-695, metropolis_hastings.py:221-226): momentum [C, D], then
  one uniform per chain for the MH test.  NUTS (nuts.py:512-529, 551-558,
  622-625, 897-900): momentum [C, D]; per depth a direction per chain; per
  leaf a uniform per chain; per depth a tree-level uniform per chain.
  """

  def __init__(self, key):
    self.key = (int(key[0]) & 0xFFFFFFFF, int(key[1]) & 0xFFFFFFFF)

  def momentum(self, shape):
    return normal(self.key, 'momentum', shape)

  def mh_uniform(self, c):
    return uniform(self.key, 'mh_uniform', c)

  def direction(self, c, depth):
    return direction(self.key, c, depth)

  def leaf_uniform(self, c, depth, leaf):
    return uniform(self.key, 'leaf_uniform', c, depth, leaf)

  def tree_uniform(self, c, depth):
    return uniform(self.key, 'tree_uniform', c, depth)


def _bits_at(key, kind, idx, depth=0, leaf=0):
  idx = np.asarray(idx, dtype=np.uint64)
  z = np.zeros_like(idx)
  return philox4x32_10(key, (idx, z + _site(kind, depth, leaf), z, z))


class OffsetDraws(PhiloxDraws):
  """Draws of a block of chains that sits inside a larger ragged batch (the
  engine's many-posterior sampler): chain i of the block is chain chain0 + i
  of the batch, and its state element d is batch element elem0 + i * D + d.
  Same streams as PhiloxDraws, addressed by those batch indices."""

  def __init__(self, key, chain0, elem0):
    super().__init__(key)
    self.chain0 = int(chain0)
    self.elem0 = int(elem0)

  def _chains(self, c):
    return self.chain0 + np.arange(c, dtype=np.uint64)

  def momentum(self, shape):
    n = int(np.prod(shape))
    o0, o1, _, _ = _bits_at(self.key, 'momentum', self.elem0 + np.arange(n, dtype=np.uint64))
    u1 = ((o0 >> np.uint32(8)).astype(np.float64) + 1.0) * 2.0 ** -24
    u2 = (o1 >> np.uint32(8)).astype(np.float64) * 2.0 ** -24
    z = np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)
    return z.astype(np.float32).reshape(shape)

  def _uniform(self, kind, c, depth=0, leaf=0):
    o0, _, _, _ = _bits_at(self.key, kind, self._chains(c), depth, leaf)
    return ((o0 >> np.uint32(8)).astype(np.float64) * 2.0 ** -24).astype(np.float32)

  def mh_uniform(self, c):
    return self._uniform('mh_uniform', c)

  def direction(self, c, depth):
    o0, _, _, _ = _bits_at(self.key, 'direction', self._chains(c), depth, 0)
    return (o0 >> np.uint32(31)).astype(np.int32)

  def leaf_uniform(self, c, depth, leaf):
    return self._uniform('leaf_uniform', c, depth, leaf)

  def tree_uniform(self, c, depth):
    return self._uniform('tree_uniform', c, depth)
