"""Free-running NUTS (gbm_nuts_run_free): every chain runs its own sequence
of NoUTurnSampler.one_step transitions (mcmc/nuts.py:321-445) with keys
step_key(seed, first_step + t) and starts the next one as soon as its own
trajectory ends.  Per chain the transitions must equal the lock-step
sampler's with the same keys:
* on a batch of multivariate-normal and hierarchical posteriors (the
  per-chain arithmetic does not depend on which other chains run), states
  and log-densities to 1e-6 and leapfrog counts and accept decisions exactly;
* on a logistic-regression target (its row-split sums depend on the batch
  size), states to 1e-5 relative on chains whose leapfrog counts agree;
* with a leaf-iteration budget, the transitions each chain completed.
"""
import numpy as np
import pytest

from tests import _problems

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')


@pytest.fixture(scope='module')
def pg():
  if not torch.cuda.is_available():
    pytest.skip('no CUDA device')
  import probability_gb300 as pg
  return pg


def _batch(pg):
  rng = np.random.default_rng(4)
  members = []
  for d, c in ((5, 16), (37, 8)):
    A = rng.standard_normal((d, d + 2)) / np.sqrt(d)
    members.append((pg.MultivariateNormalTriL(rng.normal(size=d), np.linalg.cholesky(A @ A.T)),
                    c))
  for j, c in ((8, 12), (20, 4)):
    sigma = rng.uniform(5, 20, j)
    y = 3.0 + 4.0 * rng.normal(size=j) + sigma * rng.normal(size=j)
    members.append((pg.NonCentredHierarchicalNormal(y, sigma), c))
  batch = pg.TargetBatch(members)
  q = batch.pack([torch.from_numpy((rng.normal(size=(c, t.event_dim)) * 0.5).astype(np.float32))
                  for t, c in members]).cuda()
  return batch, q


def test_free_running_equals_lock_step_on_a_batch(pg):
  batch, q = _batch(pg)
  k = pg.BatchedNoUTurnSampler(batch, step_size=[0.3, 0.1, 0.2, 0.15], max_tree_depth=8)
  kr = k.bootstrap_results(q)
  K, seed, first = 4, (5, 6), 100
  run = k.run_free(q, kr, K, seed, first_step=first)
  assert (run.transitions_done == K).all()
  qs, krs = q, kr
  for t in range(K):
    qs, krs = k.one_step(qs, krs, seed=pg._util.step_key(seed, first + t))
    np.testing.assert_array_equal(run.trace['leapfrogs_taken'][t].cpu().numpy(),
                                  krs.leapfrogs_taken.cpu().numpy())
    np.testing.assert_array_equal(run.trace['is_accepted'][t].cpu().numpy(),
                                  krs.is_accepted.cpu().numpy())
    np.testing.assert_allclose(run.all_states[t].cpu().numpy(), qs.cpu().numpy(), rtol=1e-6,
                               atol=1e-6)
    np.testing.assert_allclose(run.trace['target_log_prob'][t].cpu().numpy(),
                               krs.target_log_prob.cpu().numpy(), rtol=1e-9, atol=1e-9)
  # Every gradient evaluation of the free run is a useful leapfrog step.
  assert run.leaf_iterations <= int(run.trace['leapfrogs_taken'].sum(0).max()) + 16


def test_free_running_equals_lock_step_on_logistic_regression(pg):
  X, y, _ = _problems.logreg_data(800, 10, seed=3, scale=0.5)
  t = pg.LogisticRegression(X, y)
  C, D = 96, 10
  q = torch.from_numpy(_problems.init_state(C, D, seed=2)).cuda()
  k = pg.mcmc.NoUTurnSampler(t, step_size=0.05, max_tree_depth=7)
  kr = k.bootstrap_results(q)
  K, seed = 3, (9, 1)
  run = k.run_free(q, kr, K, seed)
  assert (run.transitions_done == K).all()
  qs, krs = q, kr
  same = np.ones(C, bool)
  for t_ in range(K):
    qs, krs = k.one_step(qs, krs, seed=pg._util.step_key(seed, t_))
    same &= run.trace['leapfrogs_taken'][t_].cpu().numpy() == krs.leapfrogs_taken.cpu().numpy()
    np.testing.assert_allclose(run.all_states[t_].cpu().numpy()[same], qs.cpu().numpy()[same],
                               rtol=1e-5, atol=1e-5)
  assert same.mean() >= 0.95


def test_free_running_budget_keeps_completed_transitions(pg):
  batch, q = _batch(pg)
  k = pg.BatchedNoUTurnSampler(batch, step_size=[0.3, 0.1, 0.2, 0.15], max_tree_depth=8)
  kr = k.bootstrap_results(q)
  K, seed = 6, (7, 7)
  full = k.run_free(q, kr, K, seed)
  cut = k.run_free(q, kr, K, seed, max_leaf_iterations=24)
  done = cut.transitions_done.cpu().numpy()
  assert done.min() < K and cut.leaf_iterations <= 24
  C = batch.chains
  offs = np.zeros(C + 1, np.int64)
  offs[1:] = np.cumsum(np.repeat(batch.member_dims, batch.member_chains))
  fs, cs = full.all_states.cpu().numpy(), cut.all_states.cpu().numpy()
  for c in range(C):
    for t in range(done[c]):
      np.testing.assert_array_equal(cs[t, offs[c]:offs[c + 1]], fs[t, offs[c]:offs[c + 1]])


def _mvn(pg, d=23, seed=8):
  rng = np.random.default_rng(seed)
  A = rng.standard_normal((d, d + 2)) / np.sqrt(d)
  return pg.MultivariateNormalTriL(rng.normal(size=d), np.linalg.cholesky(A @ A.T))


@pytest.mark.parametrize('burnin,adapt,results', [(6, 6, 14), (4, 11, 12), (12, 5, 9),
                                                  (0, 0, 10)])
def test_run_chain_free_running_draws_equal_lock_step(pg, burnin, adapt, results):
  """sample_chain with the draws past the adaptation window free-running:
  every result, the final state and the final dual-averaging state are
  bit-equal to the lock-step loop on a multivariate normal (the window may
  end before, at or after the burn-in)."""
  t = _mvn(pg)
  C = 40
  q0 = torch.from_numpy((np.random.default_rng(1).normal(size=(C, 23)) * 0.3)
                        .astype(np.float32)).cuda()
  runs = []
  for free in (False, True):
    nuts = pg.mcmc.NoUTurnSampler(t, step_size=0.3, max_tree_depth=7)
    k = pg.mcmc.DualAveragingStepSizeAdaptation(nuts, num_adaptation_steps=adapt,
                                                target_accept_prob=0.75) if adapt else nuts
    runs.append(pg.mcmc.run_chain(k, results, q0, num_burnin_steps=burnin, seed=(3, 9),
                                  free_running_draws=free))
  a, b = runs
  assert torch.equal(a.all_states, b.all_states)
  for key in a.trace:
    assert torch.equal(a.trace[key], b.trace[key]), key
  assert torch.equal(a.final_state, b.final_state)
  assert torch.equal(a.final_step_size, b.final_step_size)
  if adapt:
    assert torch.equal(a.final_da_state, b.final_da_state)


def test_run_chain_free_running_draws_logistic_regression(pg):
  """Logistic regression: the kernels' row splits depend on how many chains
  are evaluated together, so free-running and lock-step agree to rounding
  (states 1e-5 relative on chains whose leapfrog counts agree)."""
  X, y, _ = _problems.logreg_data(600, 8, seed=5, scale=0.5)
  t = pg.LogisticRegression(X, y)
  q0 = torch.from_numpy(_problems.init_state(64, 8, seed=4)).cuda()
  runs = []
  for free in (False, True):
    k = pg.mcmc.DualAveragingStepSizeAdaptation(
        pg.mcmc.NoUTurnSampler(t, step_size=0.1, max_tree_depth=7), num_adaptation_steps=8)
    runs.append(pg.mcmc.run_chain(k, 6, q0, num_burnin_steps=8, seed=(2, 2),
                                  free_running_draws=free))
  a, b = runs
  same = (a.trace['leapfrogs_taken'] == b.trace['leapfrogs_taken']).all(0).cpu().numpy()
  assert same.mean() >= 0.9
  np.testing.assert_allclose(b.all_states.cpu().numpy()[:, same], a.all_states.cpu().numpy()[:, same],
                             rtol=1e-5, atol=1e-5)
  np.testing.assert_allclose(b.final_step_size.cpu().numpy(), a.final_step_size.cpu().numpy())


def test_large_batches_compact_the_same_chains(pg):
  """Above 2048 chains the active list is built by the multi-block
  compaction.  Draws are addressed by chain index, so on a multivariate
  normal chains 0..999 of a 3000-chain batch must equal a 1000-chain batch
  bit for bit, in lock-step and free-running."""
  t = _mvn(pg, d=9, seed=3)
  rng = np.random.default_rng(6)
  q_big = torch.from_numpy((rng.normal(size=(3000, 9)) * 0.4).astype(np.float32)).cuda()
  q_small = q_big[:1000].clone()
  out = []
  for q in (q_big, q_small):
    k = pg.mcmc.NoUTurnSampler(t, step_size=0.25, max_tree_depth=8)
    kr = k.bootstrap_results(q)
    q1, kr1 = k.one_step(q, kr, seed=(4, 4))
    run = k.run_free(q, kr, 3, (4, 5))
    out.append((q1[:1000], kr1.leapfrogs_taken[:1000], run.all_states[:, :1000],
                run.trace['leapfrogs_taken'][:, :1000]))
  for a, b in zip(*out):
    assert torch.equal(a, b)
