"""Composable MetropolisHastings and dual averaging with a custom reduce_fn.

* MetropolisHastings(UncalibratedHamiltonianMonteCarlo(...)) is the
  reference's definition of HamiltonianMonteCarlo (mcmc/hmc.py:439-448): for
  the same seed it must give the fused HamiltonianMonteCarlo's results bit for
  bit, and the oracle's HMC + MH transition (mcmc/metropolis_hastings.py:
  160-254) within the parity tolerances (states 1e-5 relative).
* A proposal with a NaN log-density is rejected in-band, as safe_sum makes
  its log-accept ratio -inf (mcmc/internal/util.py:213-235).
* DualAveragingStepSizeAdaptation(reduce_fn=max) follows the reference's
  testCustomReduceFn (dual_averaging_step_size_adaptation_test.py:557-583):
  with log accept ratios log(.73), log(.76), a maximum instead of the mean
  gives the golden step size _UPDATE_01 = 10.183481 after two steps.
* reduce_log_harmonic_mean_exp (math/generic.py:387-428) is
  -reduce_logmeanexp(-x).
"""
import collections

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


def test_metropolis_hastings_of_uncalibrated_hmc_is_hmc(pg):
  X, y, _ = _problems.logreg_data(1000, 25, seed=0)
  t = pg.LogisticRegression(X, y)
  o = otargets.LogisticRegression(X, y)
  C, D = 64, 25
  q0 = torch.from_numpy(_problems.init_state(C, D)).cuda()
  mh = pg.mcmc.MetropolisHastings(
      pg.mcmc.UncalibratedHamiltonianMonteCarlo(t, step_size=0.03, num_leapfrog_steps=10))
  hmc = pg.mcmc.HamiltonianMonteCarlo(t, step_size=0.03, num_leapfrog_steps=10)
  assert mh.is_calibrated
  kr_m, kr_h = mh.bootstrap_results(q0), hmc.bootstrap_results(q0)
  qm, qh = q0, q0
  for step in range(3):
    seed = (99, step)
    prev = qm.cpu().numpy()
    lp_prev = kr_m.accepted_results.target_log_prob.cpu().numpy()
    g_prev = kr_m.accepted_results.grads_target_log_prob.cpu().numpy()
    qm, kr_m = mh.one_step(qm, kr_m, seed=seed)
    qh, kr_h = hmc.one_step(qh, kr_h, seed=seed)
    assert torch.equal(qm, qh)
    assert torch.equal(kr_m.is_accepted, kr_h.is_accepted)
    assert torch.equal(kr_m.log_accept_ratio, kr_h.log_accept_ratio)
    assert torch.equal(kr_m.accepted_results.target_log_prob,
                       kr_h.accepted_results.target_log_prob)
    assert torch.equal(kr_m.accepted_results.grads_target_log_prob,
                       kr_h.accepted_results.grads_target_log_prob)
    r = omcmc.hmc_one_step(o, prev, lp_prev, g_prev, np.float32(0.03), 10,
                           philox.PhiloxDraws(seed))
    acc = kr_m.is_accepted.cpu().numpy()
    same = acc == r.is_accepted
    assert same.sum() >= C - 1          # ties within tolerance may flip
    np.testing.assert_allclose(qm.cpu().numpy()[same], r.next_state[same], rtol=1e-5,
                               atol=1e-5)


def test_metropolis_hastings_rejects_nan_proposals(pg):
  X, y, _ = _problems.logreg_data(200, 4, seed=1)
  t = pg.LogisticRegression(X, y)
  mh = pg.mcmc.MetropolisHastings(
      pg.mcmc.UncalibratedHamiltonianMonteCarlo(t, step_size=0.1, num_leapfrog_steps=3))
  q = torch.full((8, 4), float('nan'), device='cuda')
  kr = mh.bootstrap_results(q)
  q1, kr1 = mh.one_step(q, kr, seed=(3, 3))
  assert not kr1.is_accepted.any()
  assert torch.isinf(kr1.log_accept_ratio).all() and (kr1.log_accept_ratio < 0).all()


_Fake = collections.namedtuple('FakeMHKernelResults', 'accepted_results, log_accept_ratio')
_Stepped = collections.namedtuple('FakeSteppedKernelResults', 'step_size')


def _fake_kernel(pg, log_accept_ratio):
  class FakeMH(pg.mcmc.TransitionKernel):
    """A kernel whose results only carry a step size and fixed accept ratios
    (the reference test's FakeMHKernel around FakeSteppedKernel)."""

    def __init__(self, step_size=1.0, store_parameters_in_results=True):
      self._parameters = dict(step_size=step_size,
                              store_parameters_in_results=store_parameters_in_results)

    def one_step(self, current_state, previous_kernel_results, seed=None):
      return current_state, previous_kernel_results

    def bootstrap_results(self, current_state):
      return _Fake(accepted_results=_Stepped(step_size=self._parameters['step_size']),
                   log_accept_ratio=log_accept_ratio)

  return FakeMH()


def test_dual_averaging_custom_reduce_fn_matches_reference_golden(pg):
  lar = torch.tensor([np.log(0.73), np.log(0.76)], dtype=torch.float64, device='cuda')
  kernel = pg.mcmc.DualAveragingStepSizeAdaptation(
      _fake_kernel(pg, lar), num_adaptation_steps=1,
      reduce_fn=lambda x, axis=None, keepdims=False, **_: torch.amax(x, dim=axis,
                                                                    keepdim=keepdims),
      validate_args=True)
  state = torch.zeros(2, device='cuda')
  kr = kernel.bootstrap_results(state)
  for _ in range(2):
    _, kr = kernel.one_step(state, kr)
  step = float(torch.as_tensor(kr.inner_results.accepted_results.step_size).reshape(-1)[0])
  np.testing.assert_allclose(step, 10.183481, rtol=1e-6)    # _UPDATE_01
  # The default reduction (log-mean-exp) would have lowered the step size.
  kernel_mean = pg.mcmc.DualAveragingStepSizeAdaptation(_fake_kernel(pg, lar),
                                                        num_adaptation_steps=1)
  kr = kernel_mean.bootstrap_results(state)
  for _ in range(2):
    _, kr = kernel_mean.one_step(state, kr)
  assert float(torch.as_tensor(kr.inner_results.accepted_results.step_size).reshape(-1)[0]) \
      < 10.0


def test_reduce_log_harmonic_mean_exp(pg):
  x = torch.tensor([[np.log(0.5), np.log(0.25)], [0.0, np.log(0.125)]], dtype=torch.float64)
  got = pg.mcmc.reduce_log_harmonic_mean_exp(x, axis=0).numpy()
  want = np.log(1.0 / np.mean(1.0 / np.exp(x.numpy()), axis=0))
  np.testing.assert_allclose(got, want, rtol=1e-12)
  np.testing.assert_allclose(pg.mcmc.reduce_logmeanexp(x).item(),
                             np.log(np.mean(np.exp(x.numpy()))), rtol=1e-12)
