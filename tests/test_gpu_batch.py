"""Many posteriors of uneven dimension in one sampler (TargetBatch,
BatchedNoUTurnSampler; C ABI gbm_target_batch): the batch evaluates every
member exactly as the member's own target does, one batched NUTS transition
matches the oracle run member by member on the same (batch-addressed) draws,
and CUDA-graph replay changes no bit."""
import numpy as np
import pytest

from oracle import mcmc as omcmc
from oracle import philox, targets as otargets

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')


@pytest.fixture(scope='module')
def pg():
  if not torch.cuda.is_available():
    pytest.skip('no CUDA device')
  import probability_gb300 as pg
  return pg


def _members(rng, dims_mvn=(5, 20, 70, 130), groups=(8, 12, 33), chains=(3, 5, 4, 6, 2, 7, 3)):
  """MVN members with Wishart-like covariances and hierarchical members."""
  out = []
  for d in dims_mvn:
    A = rng.normal(size=(d, d + 2)) / np.sqrt(d)
    L = np.linalg.cholesky(A @ A.T + 1e-3 * np.eye(d))
    out.append(('mvn', rng.normal(size=d), L))
  for J in groups:
    out.append(('hier', rng.normal(size=J) * 10, rng.uniform(5, 20, J)))
  return out, list(chains[:len(out)])


def _build(pg, spec, chains, stream=None):
  eng, orc = [], []
  for s in spec:
    if s[0] == 'mvn':
      eng.append(pg.MultivariateNormalTriL(s[1], s[2]))
      orc.append(otargets.MultivariateNormalTriL(s[1], s[2]))
    else:
      eng.append(pg.NonCentredHierarchicalNormal(s[1], s[2]))
      orc.append(otargets.NonCentredHierarchicalNormal(s[1], s[2]))
  return pg.TargetBatch(list(zip(eng, chains)), stream=stream), eng, orc


def _init(rng, batch):
  return [(rng.normal(size=(c, t.event_dim)) * 0.5).astype(np.float32)
          for t, c in zip(batch.members, batch.member_chains)]


def test_batch_matches_member_targets(pg):
  rng = np.random.default_rng(0)
  spec, chains = _members(rng)
  batch, eng, _ = _build(pg, spec, chains)
  init = _init(rng, batch)
  lp, g = batch.log_prob_and_grad(batch.pack([torch.from_numpy(x) for x in init]).cuda())
  parts = batch.unpack(g)
  c0 = 0
  for t, x in enumerate(init):
    lp_t, g_t = eng[t].log_prob_and_grad(torch.from_numpy(x).cuda())
    np.testing.assert_allclose(lp[c0:c0 + x.shape[0]].cpu().numpy(), lp_t.cpu().numpy(),
                               rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(parts[t].cpu().numpy(), g_t.cpu().numpy(), rtol=1e-5, atol=1e-5)
    c0 += x.shape[0]
  sched = batch.schedule()
  assert set(sched.values()) <= {0, 32, 64}


def test_batched_nuts_transition_matches_oracle_per_member(pg):
  rng = np.random.default_rng(1)
  spec, chains = _members(rng)
  batch, _, orc = _build(pg, spec, chains)
  init = _init(rng, batch)
  steps = [0.2, 0.1, 0.05, 0.04, 0.15, 0.1, 0.05]
  k = pg.BatchedNoUTurnSampler(batch, steps[:len(init)], max_tree_depth=6)
  q = batch.pack([torch.from_numpy(x) for x in init]).cuda()
  kr = k.bootstrap_results(q)
  q1, kr1 = k.one_step(q, kr, seed=(5, 6))
  key = pg._util.sanitize_seed((5, 6))
  out = batch.unpack(q1)
  lf = kr1.leapfrogs_taken.cpu().numpy()
  c0 = 0
  for t, x in enumerate(init):
    lp, g = orc[t](x.astype(np.float64))
    r = omcmc.nuts_one_step(orc[t], x, lp, g, np.float32(steps[t]),
                            philox.OffsetDraws(key, batch.chain_begin[t], batch.elem_begin[t]), 6)
    n = x.shape[0]
    same = lf[c0:c0 + n] == r.leapfrogs_taken
    assert same.sum() >= n - 1, (t, lf[c0:c0 + n], r.leapfrogs_taken)
    np.testing.assert_allclose(out[t].cpu().numpy()[same], r.next_state[same], rtol=1e-4,
                               atol=1e-4)
    c0 += n


def test_graph_replay_is_bit_identical_to_per_leaf_launches(pg):
  """Graph replay of batches of leaves and leaf-by-leaf launches give the
  same bits."""
  rng = np.random.default_rng(2)
  spec, chains = _members(rng, dims_mvn=(6, 40), groups=(10,), chains=(8, 4, 6))
  batch, _, _ = _build(pg, spec, chains)
  init = _init(rng, batch)
  q0 = batch.pack([torch.from_numpy(x) for x in init]).cuda()
  k = pg.BatchedNoUTurnSampler(batch, [0.1, 0.05, 0.1], max_tree_depth=8)
  kr = k.bootstrap_results(q0)
  q, states = q0, []
  for i in range(4):
    q, kr = k.one_step(q, kr, seed=(9, i))
    states.append(q.clone())
  # The same sampler launching leaf by leaf (no graphs), on the legacy stream.
  batch2, _, _ = _build(pg, spec, chains, stream=torch.cuda.default_stream())
  k2 = pg.BatchedNoUTurnSampler(batch2, [0.1, 0.05, 0.1], max_tree_depth=8, use_graphs=False)
  kr2 = k2.bootstrap_results(q0)
  q2 = q0
  for i in range(4):
    q2, kr2 = k2.one_step(q2, kr2, seed=(9, i))
    assert torch.equal(q2, states[i])


def test_preconditioned_batched_transition_matches_oracle(pg):
  """A ragged inverse mass (one value per state element) in the batched
  sampler equals the oracle's preconditioned NUTS member by member."""
  rng = np.random.default_rng(4)
  spec, chains = _members(rng, dims_mvn=(9, 33), groups=(10,), chains=(5, 4, 6))
  batch, _, orc = _build(pg, spec, chains)
  init = _init(rng, batch)
  steps = [0.1, 0.05, 0.1]
  k = pg.BatchedNoUTurnSampler(batch, steps, max_tree_depth=6)
  inv_mass = [rng.uniform(0.3, 2.0, size=x.shape).astype(np.float32) for x in init]
  k.set_inverse_mass(batch.pack([torch.from_numpy(v) for v in inv_mass]).cuda())
  q = batch.pack([torch.from_numpy(x) for x in init]).cuda()
  kr = k.bootstrap_results(q)
  q1, kr1 = k.one_step(q, kr, seed=(2, 3))
  out = batch.unpack(q1)
  lf = kr1.leapfrogs_taken.cpu().numpy()
  key = pg._util.sanitize_seed((2, 3))
  c0 = 0
  for t, x in enumerate(init):
    lp, g = orc[t](x.astype(np.float64))
    r = omcmc.nuts_one_step(orc[t], x, lp, g, np.float32(steps[t]),
                            philox.OffsetDraws(key, batch.chain_begin[t], batch.elem_begin[t]), 6,
                            inv_mass=inv_mass[t])
    n = x.shape[0]
    same = lf[c0:c0 + n] == r.leapfrogs_taken
    assert same.sum() >= n - 1
    np.testing.assert_allclose(out[t].cpu().numpy()[same], r.next_state[same], rtol=1e-4,
                               atol=1e-4)
    c0 += n
