"""TransformedTransitionKernel (mcmc/transformed_kernel.py:165) on the
engine: the transformed target (gbm_target_transformed) against the FP64
oracle, and a TransformedTransitionKernel(NoUTurnSampler) transition against
the oracle NUTS on the transformed oracle target with the same draws."""
import numpy as np
import pytest

from oracle import mcmc as omcmc
from oracle import philox, targets as otargets
from tests import _problems

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')


@pytest.fixture(scope='module')
def pg():
  if not torch.cuda.is_available():
    pytest.skip('no CUDA device')
  import probability_gb300 as pg
  return pg


def test_transformed_target_matches_oracle(pg):
  from probability_gb300.mcmc.transformed_kernel import TransformedTarget
  X, y, _ = _problems.logreg_data(800, 7, seed=4, scale=0.5)
  codes = [0, 1, 2, 3, 1, 2, 0]
  t = TransformedTarget(pg.LogisticRegression(X, y), codes)
  o = otargets.TransformedTarget(otargets.LogisticRegression(X, y), codes)
  x = (np.random.default_rng(5).normal(size=(33, 7)) * 0.6).astype(np.float32)
  lp, g = t.log_prob_and_grad(torch.from_numpy(x).cuda())
  lp_o, g_o = o(x)
  np.testing.assert_allclose(lp.cpu().numpy(), lp_o, rtol=2e-6, atol=1e-4)
  np.testing.assert_allclose(g.cpu().numpy(), g_o, rtol=1e-4, atol=1e-3)


def test_transformed_nuts_transition_matches_oracle(pg):
  """Eight-schools-style use (nuts_test.py:525-529): a positive scale
  sampled through Exp, here on a logistic regression's coefficients."""
  X, y, _ = _problems.logreg_data(600, 5, seed=6, scale=0.5)
  bij = pg.bijectors.Softplus()
  inner = pg.mcmc.NoUTurnSampler(pg.LogisticRegression(X, y), step_size=0.05, max_tree_depth=6)
  k = pg.mcmc.TransformedTransitionKernel(inner, bij)
  C = 24
  init = torch.from_numpy((np.random.default_rng(1).uniform(0.2, 1.5, size=(C, 5)))
                          .astype(np.float32)).cuda()
  kr = k.bootstrap_results(init)
  xt = kr.transformed_state
  np.testing.assert_allclose(bij.forward(xt).cpu().numpy(), init.cpu().numpy(), rtol=1e-5)
  q1, kr1 = k.one_step(init, kr, seed=(3, 9))
  assert type(kr1).__name__ == 'TransformedTransitionKernelResults'
  np.testing.assert_allclose(q1.cpu().numpy(), bij.forward(kr1.transformed_state).cpu().numpy(),
                             rtol=1e-6)
  o = otargets.TransformedTarget(otargets.LogisticRegression(X, y), [2] * 5)
  x0 = xt.cpu().numpy()
  lp, g = o(x0.astype(np.float64))
  r = omcmc.nuts_one_step(o, x0, lp, g, np.float32(0.05), philox.PhiloxDraws((3, 9)), 6)
  lf = kr1.inner_results.leapfrogs_taken.cpu().numpy()
  same = lf == r.leapfrogs_taken
  assert same.sum() >= C - 1
  np.testing.assert_allclose(kr1.transformed_state.cpu().numpy()[same], r.next_state[same],
                             rtol=1e-4, atol=1e-4)
  # The result is in the constrained space.
  assert (q1 > 0).all()


def test_transformed_kernel_contract(pg):
  X, y, _ = _problems.logreg_data(200, 3, seed=2)
  k = pg.mcmc.TransformedTransitionKernel(
      pg.mcmc.HamiltonianMonteCarlo(pg.LogisticRegression(X, y), step_size=0.05,
                                    num_leapfrog_steps=3), pg.bijectors.Exp())
  assert k.is_calibrated
  with pytest.raises(ValueError):
    k.bootstrap_results()
  x = torch.ones(4, 3).cuda()
  kr = k.bootstrap_results(transformed_init_state=x)
  q, kr = k.one_step(None, kr, seed=(1, 1))
  assert q.shape == (4, 3) and (q > 0).all()
