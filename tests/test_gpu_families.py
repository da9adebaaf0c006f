"""Multivariate-normal and non-centred hierarchical targets against the FP64
oracle: log-density and gradient, NUTS transitions on identical draws, and
posterior moments of a long run against the exact ones.

Tolerances: log-density rtol 1e-5 (+1e-3 absolute), gradient 1e-4 x
max|grad| + rtol 1e-4; transition states rtol/atol 1e-5 (FP32 state).
"""
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


def _wishart_mvn(d, seed):
  """Covariance ~ Wishart(d + 2, I/d) as in the batched-posterior workload."""
  rng = np.random.default_rng(seed)
  A = rng.normal(size=(d, d + 2)) / np.sqrt(d)
  cov = A @ A.T
  L = np.linalg.cholesky(cov)
  return rng.normal(size=d), L


def _hier(J, seed):
  rng = np.random.default_rng(seed)
  mu, tau = rng.normal() * 5, abs(rng.standard_cauchy()) * 5
  sigma = rng.uniform(5, 20, J)
  y = mu + tau * rng.normal(size=J) + sigma * rng.normal(size=J)
  return y.astype(np.float32), sigma.astype(np.float32)


def _check(t, o, q):
  lp, g = t.log_prob_and_grad(torch.from_numpy(q).cuda())
  lp_o, g_o = o(q)
  np.testing.assert_allclose(lp.cpu().numpy(), lp_o, rtol=1e-5, atol=1e-3)
  np.testing.assert_allclose(g.cpu().numpy(), g_o, rtol=1e-4, atol=1e-4 * np.abs(g_o).max())


@pytest.mark.parametrize('d,c', [(8, 32), (65, 70), (300, 129), (2048, 40)])
def test_mvn_log_prob_and_grad(pg, d, c):
  """Wishart(D+2, I/D) covariances are badly conditioned at large D; FP32
  errors of u = L^-1 (x - loc) grow like eps * cond(L), so the stated
  tolerances scale with cond(L): log-density rtol 4e-7 cond(L) (at least
  1e-5), gradient 4e-7 cond(L) max|grad| (at least 1e-4 max|grad|)."""
  loc, L = _wishart_mvn(d, seed=d)
  t = pg.MultivariateNormalTriL(loc, L)
  o = otargets.MultivariateNormalTriL(loc, L)
  q = (loc + np.random.default_rng(c).normal(size=(c, d)) @ L.T * 0.7).astype(np.float32)
  cond = np.linalg.cond(L)
  lp, g = t.log_prob_and_grad(torch.from_numpy(q).cuda())
  lp_o, g_o = o(q)
  np.testing.assert_allclose(lp.cpu().numpy(), lp_o, rtol=max(1e-5, 4e-7 * cond), atol=1e-3)
  np.testing.assert_allclose(g.cpu().numpy(), g_o, rtol=0,
                             atol=max(1e-4, 4e-7 * cond) * np.abs(g_o).max())


@pytest.mark.parametrize('J,c', [(8, 32), (100, 70), (512, 33)])
def test_hierarchical_log_prob_and_grad(pg, J, c):
  y, sigma = _hier(J, seed=J)
  t = pg.NonCentredHierarchicalNormal(y, sigma)
  o = otargets.NonCentredHierarchicalNormal(y, sigma)
  rng = np.random.default_rng(c)
  q = np.concatenate([rng.normal(size=(c, 1)) * 3, rng.normal(size=(c, 1)),
                      rng.normal(size=(c, J))], 1).astype(np.float32)
  _check(t, o, q)


@pytest.mark.parametrize('family', ['mvn', 'hier'])
def test_nuts_transition_matches_oracle(pg, family):
  if family == 'mvn':
    loc, L = _wishart_mvn(20, seed=3)
    t, o = pg.MultivariateNormalTriL(loc, L), otargets.MultivariateNormalTriL(loc, L)
    q0 = (loc + np.random.default_rng(0).normal(size=(40, 20)) * 0.1).astype(np.float32)
    eps = 0.05
  else:
    y, sigma = _hier(8, seed=4)
    t, o = pg.NonCentredHierarchicalNormal(y, sigma), otargets.NonCentredHierarchicalNormal(y, sigma)
    q0 = (np.random.default_rng(1).normal(size=(40, 10)) * 0.5).astype(np.float32)
    eps = 0.2
  k = pg.mcmc.NoUTurnSampler(t, step_size=eps, max_tree_depth=8)
  q = torch.from_numpy(q0).cuda()
  kr = k.bootstrap_results(q)
  q1, kr1 = k.one_step(q, kr, seed=(6, 6))
  r = omcmc.nuts_one_step(o, q0, kr.target_log_prob.cpu().numpy(),
                          kr.grads_target_log_prob.cpu().numpy(), np.float32(eps),
                          philox.PhiloxDraws((6, 6)), 8)
  same = kr1.leapfrogs_taken.cpu().numpy() == r.leapfrogs_taken
  assert same.sum() >= len(same) - 1
  np.testing.assert_allclose(q1.cpu().numpy()[same], r.next_state[same], rtol=1e-5, atol=1e-5)


def test_nuts_mvn_posterior_moments(pg):
  """A correlated 10-D Gaussian: NUTS + dual averaging draws match the exact
  mean and covariance within Monte Carlo error; split R-hat < 1.01."""
  from oracle import diagnostics
  loc, L = _wishart_mvn(10, seed=7)
  cov = L @ L.T
  t = pg.MultivariateNormalTriL(loc, L)
  k = pg.mcmc.DualAveragingStepSizeAdaptation(
      pg.mcmc.NoUTurnSampler(t, step_size=0.1, max_tree_depth=8), num_adaptation_steps=150,
      target_accept_prob=0.8)
  q0 = torch.from_numpy((loc + np.random.default_rng(2).normal(size=(128, 10))).astype(np.float32))
  run = pg.mcmc.run_chain(k, 400, q0.cuda(), num_burnin_steps=200, seed=(3, 3))
  d = run.all_states.cpu().numpy().astype(np.float64)
  rhat = diagnostics.potential_scale_reduction(d, split_chains=True)
  assert np.all(rhat < 1.01), rhat.max()
  ess = diagnostics.effective_sample_size(d, filter_beyond_positive_pairs=True).sum(0)
  mean = d.reshape(-1, 10).mean(0)
  se = np.sqrt(np.diag(cov) / ess)
  assert np.all(np.abs(mean - loc) < 4.5 * se), (np.abs(mean - loc) / se).max()
  np.testing.assert_allclose(np.cov(d.reshape(-1, 10).T), cov, atol=0.15 * np.abs(cov).max())
