"""PreconditionedNoUTurnSampler and DiagonalMassMatrixAdaptation
(experimental/mcmc/preconditioned_nuts.py:169,
diagonal_mass_matrix_adaptation.py:73) on the engine: a preconditioned
transition matches the oracle with the same inverse mass and draws, the
identity mass gives NoUTurnSampler's bits, and adaptation recovers the
marginal variances of an ill-conditioned Gaussian."""
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


def test_preconditioned_transition_matches_oracle(pg):
  from probability_gb300.experimental.mcmc import DiagonalMomentum, PreconditionedNoUTurnSampler
  X, y, _ = _problems.logreg_data(800, 12, seed=3, scale=0.5)
  t = pg.LogisticRegression(X, y)
  o = otargets.LogisticRegression(X, y)
  v = np.random.default_rng(0).uniform(0.2, 3.0, 12).astype(np.float32)
  C = 40
  q = torch.from_numpy(_problems.init_state(C, 12, seed=2)).cuda()
  k = PreconditionedNoUTurnSampler(t, step_size=0.04, max_tree_depth=7,
                                   momentum_distribution=DiagonalMomentum(torch.from_numpy(v).cuda()))
  kr = k.bootstrap_results(q)
  mism = 0
  for s in range(3):
    q_in = q.cpu().numpy()
    l_in = kr.target_log_prob.cpu().numpy()
    g_in = kr.grads_target_log_prob.cpu().numpy()
    q, kr = k.one_step(q, kr, seed=(7, s))
    r = omcmc.nuts_one_step(o, q_in, l_in, g_in, np.float32(0.04), philox.PhiloxDraws((7, s)), 7,
                            inv_mass=v)
    same = kr.leapfrogs_taken.cpu().numpy() == r.leapfrogs_taken
    mism += int((~same).sum())
    np.testing.assert_allclose(q.cpu().numpy()[same], r.next_state[same], rtol=1e-4, atol=1e-4)
    np.testing.assert_allclose(kr.energy.cpu().numpy()[same], r.energy[same], rtol=1e-6, atol=2e-3)
    assert type(kr).__name__ == 'PreconditionedNUTSKernelResults'
  assert mism <= 2


def test_identity_mass_gives_nuts_bits(pg):
  from probability_gb300.experimental.mcmc import PreconditionedNoUTurnSampler
  X, y, _ = _problems.logreg_data(500, 6, seed=4, scale=0.5)
  t = pg.LogisticRegression(X, y)
  q0 = torch.from_numpy(_problems.init_state(16, 6, seed=5)).cuda()
  a = pg.mcmc.NoUTurnSampler(t, step_size=0.05, max_tree_depth=6)
  b = PreconditionedNoUTurnSampler(t, step_size=0.05, max_tree_depth=6)
  ka, kb = a.bootstrap_results(q0), b.bootstrap_results(q0)
  qa, qb = q0, q0
  for s in range(3):
    qa, ka = a.one_step(qa, ka, seed=(1, s))
    qb, kb = b.one_step(qb, kb, seed=(1, s))
  assert torch.equal(qa, qb)
  assert torch.equal(ka.leapfrogs_taken, kb.leapfrogs_taken)


def test_mass_matrix_adaptation_learns_marginal_variances(pg):
  from probability_gb300.experimental.mcmc import (DiagonalMassMatrixAdaptation,
                                                   PreconditionedNoUTurnSampler)
  from probability_gb300.experimental.stats import RunningVariance
  d = 8
  scales = np.geomspace(0.05, 5.0, d)
  target = pg.MultivariateNormalTriL(np.zeros(d), np.diag(scales))
  inner = pg.mcmc.DualAveragingStepSizeAdaptation(
      PreconditionedNoUTurnSampler(target, step_size=0.01, max_tree_depth=8),
      num_adaptation_steps=150, target_accept_prob=0.8)
  k = DiagonalMassMatrixAdaptation(inner, RunningVariance.from_shape((d,)))
  q = torch.from_numpy((np.random.default_rng(3).normal(size=(128, d)) * scales * 0.5)
                       .astype(np.float32)).cuda()
  kr = k.bootstrap_results(q)
  for s in range(200):
    q, kr = k.one_step(q, kr, seed=(11, s))
  var = kr.running_variance.variance().cpu().numpy()
  ratio = var / scales ** 2
  assert np.all(ratio > 0.5) and np.all(ratio < 2.0), ratio
