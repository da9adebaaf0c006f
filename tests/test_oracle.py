"""The oracle pinned against the reference's golden vectors and KATs (CPU)."""
import json
import os

import numpy as np
import pytest

from oracle import diagnostics, mcmc, philox, targets


def test_philox_known_answers(golden_dir):
  for case in json.load(open(os.path.join(golden_dir, 'philox_kat.json'))):
    out = philox.philox4x32_10(case['key'], [np.array([c]) for c in case['ctr']])
    assert [int(o[0]) for o in out] == case['out']


def test_nuts_instruction_tables_match_reference(golden_dir):
  # nuts_test.py:191-215 pins depth 4; the fixture holds the reference's own
  # generator output for depths 1..12.
  tables = json.load(open(os.path.join(golden_dir, 'nuts_instructions.json')))
  for depth, t in tables.items():
    w, r = mcmc.write_read_instruction(int(depth))
    assert w.tolist() == t['write']
    assert r.tolist() == t['read']
  w, r = mcmc.write_read_instruction(4)
  assert w.tolist() == [0, 4, 1, 4, 1, 4, 2, 4, 1, 4, 2, 4, 2, 4, 3, 4]


def test_instruction_dummy_slot_never_read():
  for depth in range(1, 11):
    w, r = mcmc.write_read_instruction(depth)
    assert r.max() <= w.max()          # the dummy slot index is never in a range
    for j in range(1 << depth):
      for i in range(r[j, 0], r[j, 1]):
        assert i != w.max()


def test_dual_averaging_golden_constants(golden_dir):
  g = json.load(open(os.path.join(golden_dir, 'dual_averaging.json')))
  for case in g['cases']:
    da = mcmc.DualAveraging(1.0, num_adaptation_steps=10)
    da.update(np.log(g['target'] + case['err']))
    np.testing.assert_allclose(da.new_step_size, case['expected'], rtol=1e-6)


def test_dual_averaging_list_step_and_chain_target():
  # dual_averaging_step_size_adaptation_test.py:177-198 and :262-290
  da = mcmc.DualAveraging(np.array([0.1, 0.2, 0.3]), num_adaptation_steps=1)
  for _ in range(2):
    da.update(np.log([0.74, 0.76, 0.76]))
  exp = np.exp(np.log(10 * np.array([0.1, 0.2, 0.3])) - np.array([0.01, -0.01, -0.01]) / (11 * 0.05))
  np.testing.assert_allclose(da.new_step_size, exp, rtol=1e-6)
  da = mcmc.DualAveraging(np.array([0.1, 0.2]), num_adaptation_steps=1,
                          target_accept_prob=np.array([0.7, 0.8]))
  for _ in range(2):
    da.update(np.log([0.74, 0.76]))
  exp = np.exp(np.log(10 * np.array([0.1, 0.2])) - np.array([-0.04, 0.04]) / (11 * 0.05))
  np.testing.assert_allclose(da.new_step_size, exp, rtol=1e-6)


def test_dual_averaging_recovers_from_nan():
  da = mcmc.DualAveraging(0.1, num_adaptation_steps=1)
  for _ in range(2):
    da.update(np.nan)
  assert np.isfinite(da.new_step_size)


def _logreg(n=200, d=5, seed=0):
  rng = np.random.default_rng(seed)
  X = np.concatenate([np.ones((n, 1)), rng.normal(size=(n, d - 1))], 1)
  beta = rng.normal(size=d)
  y = (rng.uniform(size=n) < 1 / (1 + np.exp(-X @ beta))).astype(np.float64)
  return targets.LogisticRegression(X, y)


def _fd_check(t, x, h=1e-6):
  lp, g = t(x)
  num = np.zeros_like(x)
  for j in range(x.shape[1]):
    e = np.zeros_like(x)
    e[:, j] = h
    num[:, j] = (t(x + e)[0] - t(x - e)[0]) / (2 * h)
  np.testing.assert_allclose(g, num, rtol=1e-5, atol=1e-5)


def test_target_gradients_finite_difference():
  rng = np.random.default_rng(1)
  _fd_check(_logreg(), rng.normal(size=(3, 5)))
  L = np.tril(rng.normal(size=(4, 4))) + 3 * np.eye(4)
  _fd_check(targets.MultivariateNormalTriL(rng.normal(size=4), L), rng.normal(size=(3, 4)))
  h = targets.NonCentredHierarchicalNormal(rng.normal(size=6) * 10, rng.uniform(5, 20, 6))
  _fd_check(h, rng.normal(size=(3, 8)))


def test_target_gradients_torch_autograd():
  torch = pytest.importorskip('torch')
  rng = np.random.default_rng(2)
  t = _logreg()
  b = rng.normal(size=(4, 5))
  bt = torch.tensor(b, requires_grad=True)
  X = torch.tensor(t.X)
  y = torch.tensor(t.y)
  z = bt @ X.T
  lp = (torch.distributions.Bernoulli(logits=z).log_prob(y).sum(-1)
        + torch.distributions.Normal(0., 1.).log_prob(bt).sum(-1))
  lp.sum().backward()
  lp_o, g_o = t(b)
  np.testing.assert_allclose(lp.detach().numpy(), lp_o, rtol=1e-12)
  np.testing.assert_allclose(bt.grad.numpy(), g_o, rtol=1e-10, atol=1e-12)


def test_hmc_nan_proposal_is_rejected():
  # hmc_test.py:398-431: a NaN log-prob proposal leaves the state unchanged.
  def bad(x):
    return np.full(x.shape[0], np.nan), np.zeros_like(x)
  def good(x):
    return -0.5 * np.sum(x * x, -1), -x
  x = np.ones((4, 3))
  lp, g = good(x)
  r = mcmc.hmc_one_step(bad, x, lp, g, 0.1, 3, philox.PhiloxDraws((1, 2)))
  assert not r.is_accepted.any()
  assert np.all(r.log_accept_ratio == -np.inf)
  np.testing.assert_array_equal(r.next_state, x)


def test_nuts_nan_target_diverges_and_keeps_state():
  calls = {'n': 0}
  def tgt(x):
    calls['n'] += 1
    return np.full(x.shape[0], np.nan), np.full_like(x, np.nan)
  x = np.zeros((5, 2))
  r = mcmc.nuts_one_step(tgt, x, np.zeros(5), np.zeros((5, 2)), 0.1,
                         philox.PhiloxDraws((3, 4)), max_tree_depth=5)
  assert r.has_divergence.all()
  assert not r.is_accepted.any()
  np.testing.assert_array_equal(r.next_state, x)
  assert np.all(r.leapfrogs_taken == 1)


def test_nuts_reproducible_and_seed_dependent():
  t = _logreg()
  x = np.random.default_rng(0).normal(size=(6, 5)) * 0.1
  lp, g = t(x)
  a = mcmc.nuts_one_step(t, x, lp, g, 0.05, philox.PhiloxDraws((7, 8)), 6)
  b = mcmc.nuts_one_step(t, x, lp, g, 0.05, philox.PhiloxDraws((7, 8)), 6)
  c = mcmc.nuts_one_step(t, x, lp, g, 0.05, philox.PhiloxDraws((7, 9)), 6)
  np.testing.assert_array_equal(a.next_state, b.next_state)
  assert not np.array_equal(a.next_state, c.next_state)


def test_nuts_chain_transitions_do_not_depend_on_the_batch():
  """The lock-step NUTS transition (nuts.py:541-711: finished chains only
  idle under the batch's masks) gives every chain the transition it would
  have alone with the same draws -- the property free-running NUTS uses to
  let each chain start its next transition on its own.  A batch of 5 chains
  over 3 transitions equals each chain run alone with its draws addressed
  as part of the batch (OffsetDraws): the same trajectory lengths exactly,
  states and log-densities to 1e-12 (NumPy's BLAS rounds a 5-row product
  and a 1-row product differently, in the last bit)."""
  rng = np.random.default_rng(3)
  D, C = 4, 5
  A = rng.normal(size=(D, D + 2)) / np.sqrt(D)
  t = targets.MultivariateNormalTriL(rng.normal(size=D), np.linalg.cholesky(A @ A.T))
  x = rng.normal(size=(C, D)) * 0.5
  eps = np.array([0.2, 0.3, 0.25, 0.15, 0.35])
  lp, g = t(x)
  batch = [(x, lp, g)]
  alone = [[(x[c:c + 1], lp[c:c + 1], g[c:c + 1])] for c in range(C)]
  for step in range(3):
    key = (11, step)
    q, l, gr = batch[-1]
    r = mcmc.nuts_one_step(t, q, l, gr, eps, philox.PhiloxDraws(key), 6)
    batch.append((r.next_state, r.target_log_prob, r.grads_target_log_prob))
    for c in range(C):
      qc, lc, gc = alone[c][-1]
      rc = mcmc.nuts_one_step(t, qc, lc, gc, eps[c:c + 1],
                              philox.OffsetDraws(key, chain0=c, elem0=c * D), 6)
      alone[c].append((rc.next_state, rc.target_log_prob, rc.grads_target_log_prob))
      np.testing.assert_array_equal(rc.leapfrogs_taken[0], r.leapfrogs_taken[c])
      np.testing.assert_allclose(rc.next_state[0], r.next_state[c], rtol=1e-12, atol=1e-12)
      np.testing.assert_allclose(rc.target_log_prob[0], r.target_log_prob[c], rtol=1e-12)


def test_leapfrog_energy_conservation():
  # leapfrog_integrator_test.py:48-73: 1000 steps, rtol 0.02 on energy.
  def tgt(x):
    return -0.5 * np.sum(x * x, -1), -x
  rng = np.random.default_rng(3)
  q = rng.normal(size=(2, 10))
  p = rng.normal(size=(2, 10))
  lp, g = tgt(q)
  h0 = lp - 0.5 * np.sum(p * p, -1)
  for _ in range(100):
    p, q, lp, g = mcmc.leapfrog(tgt, p, q, lp, g, 0.1, 10)
  h1 = lp - 0.5 * np.sum(p * p, -1)
  np.testing.assert_allclose(h1, h0, rtol=0.02)


def _mvn2d():
  cov = np.array([[1.0, 0.8], [0.8, 1.0]])
  L = np.linalg.cholesky(cov)
  return targets.MultivariateNormalTriL(np.array([1.0, -2.0]), L), cov


def test_hmc_mvn_moments():
  # hmc_test.py:494-542 pattern: correlated 2-D MVN, mean/cov tolerances.
  t, cov = _mvn2d()
  x = np.zeros((64, 2))
  lp, g = t(x)
  draws = []
  acc = []
  for s in range(600):
    r = mcmc.hmc_one_step(t, x, lp, g, 0.25, 4, philox.PhiloxDraws((11, s)))
    x, lp, g = r.next_state, r.target_log_prob, r.grads_target_log_prob
    acc.append(r.is_accepted.mean())
    if s >= 100:
      draws.append(x)
  d = np.concatenate(draws)
  np.testing.assert_allclose(d.mean(0), [1.0, -2.0], atol=0.06)
  np.testing.assert_allclose(np.cov(d.T), cov, atol=0.08)
  assert 0.5 < np.mean(acc) <= 1.0


def test_nuts_mvn_moments_and_ess():
  # nuts_test.py:306-356 pattern (mean/cov) plus ESS/R-hat on the draws.
  t, cov = _mvn2d()
  x = np.zeros((32, 2))
  lp, g = t(x)
  draws = []
  for s in range(1000):
    r = mcmc.nuts_one_step(t, x, lp, g, 0.3, philox.PhiloxDraws((5, s)), 6)
    x, lp, g = r.next_state, r.target_log_prob, r.grads_target_log_prob
    if s >= 100:
      draws.append(x)
  d = np.stack(draws)                                   # [n, C, 2]
  flat = d.reshape(-1, 2)
  np.testing.assert_allclose(flat.mean(0), [1.0, -2.0], atol=0.06)
  np.testing.assert_allclose(np.cov(flat.T), cov, atol=0.1)
  ess = diagnostics.effective_sample_size(d).sum(0)
  assert np.all(ess > 4000)
  rhat = diagnostics.potential_scale_reduction(d, split_chains=True)
  assert np.all(rhat < 1.01)


def test_ess_iid_and_ar1():
  rng = np.random.default_rng(4)
  x = rng.normal(size=(2000, 8))
  ess = diagnostics.effective_sample_size(x)
  assert np.all(np.abs(ess / 2000 - 1) < 0.2)
  rho = 0.9
  y = np.zeros((4000, 8))
  for t in range(1, 4000):
    y[t] = rho * y[t - 1] + rng.normal(size=8) * np.sqrt(1 - rho ** 2)
  ess = diagnostics.effective_sample_size(y, filter_beyond_positive_pairs=True)
  expected = 4000 * (1 - rho) / (1 + rho)
  assert np.all(np.abs(ess / expected - 1) < 0.35)
  ess_cc = diagnostics.effective_sample_size(y[:, :, None], cross_chain_dims=1)
  assert ess_cc.shape == (1,)


def test_sample_chain_step_count():
  assert mcmc.num_transitions(10, 5, 2) == 5 + 1 + 9 * 3


def test_transformed_target_gradient_finite_difference():
  """TransformedTarget (transformed_kernel.py:63-95): log p(f(x)) + log|f'(x)|
  and its gradient, for every bijector, against central differences."""
  rng = np.random.default_rng(11)
  X = rng.normal(size=(40, 6))
  X[:, 0] = 1
  y = (rng.uniform(size=40) < 0.5).astype(float)
  t = targets.TransformedTarget(targets.LogisticRegression(X, y), [0, 1, 2, 3, 1, 0])
  x = rng.normal(size=(3, 6)) * 0.7
  lp, g = t(x)
  eps = 1e-6
  for d in range(6):
    e = np.zeros(6)
    e[d] = eps
    np.testing.assert_allclose(g[:, d], (t(x + e)[0] - t(x - e)[0]) / (2 * eps), rtol=1e-6,
                               atol=1e-6)


def test_running_variance_merges_batches():
  """experimental/stats RunningVariance: batched (Chan) updates equal the
  variance of all samples."""
  torch = pytest.importorskip('torch')
  from probability_gb300.experimental.stats import RunningVariance
  x = torch.from_numpy(np.random.default_rng(0).normal(size=(97, 4)) * [1, 2, 3, 4])
  rv = RunningVariance.from_shape((4,))
  for a, b in [(0, 10), (10, 11), (11, 60), (60, 97)]:
    rv = rv.update(x[a:b], axis=0)
  np.testing.assert_allclose(rv.variance().numpy(), x.var(0, unbiased=False).numpy(), rtol=1e-12)
