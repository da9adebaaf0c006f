"""Device-resident sample_chain loops (gbm_*_sample_chain) against the
Python-driven sample_chain over the same kernels and step keys: identical
bits, since both run the same deterministic kernels on the same draws."""
import numpy as np
import pytest

from oracle import diagnostics
from tests import _problems

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')


@pytest.fixture(scope='module')
def pg():
  if not torch.cuda.is_available():
    pytest.skip('no CUDA device')
  import probability_gb300 as pg
  return pg


def _target(pg, n=800, d=10, precision='fp32'):
  X, y, beta = _problems.logreg_data(n, d, seed=31, scale=0.5)
  return pg.LogisticRegression(X, y, precision=precision), beta


def test_native_nuts_da_loop_equals_python_loop(pg):
  t, _ = _target(pg)
  q0 = torch.from_numpy(_problems.init_state(24, 10, seed=2)).cuda()
  make = lambda: pg.mcmc.DualAveragingStepSizeAdaptation(
      pg.mcmc.NoUTurnSampler(t, step_size=0.1, max_tree_depth=7), num_adaptation_steps=5,
      target_accept_prob=0.8)
  native = pg.mcmc.sample_chain(6, q0, kernel=make(), num_burnin_steps=3,
                                num_steps_between_results=1, trace_fn=None, seed=(4, 2))
  python = pg.mcmc.sample_chain(6, q0, kernel=make(), num_burnin_steps=3,
                                num_steps_between_results=1, trace_fn=lambda s, kr: (),
                                seed=(4, 2)).all_states
  assert native.shape == (6, 24, 10)
  assert torch.equal(native, python)


def test_native_hmc_loop_equals_python_loop(pg):
  t, _ = _target(pg, 500, 6)
  q0 = torch.from_numpy(_problems.init_state(16, 6, seed=5)).cuda()
  k = pg.mcmc.HamiltonianMonteCarlo(t, step_size=0.05, num_leapfrog_steps=4)
  native = pg.mcmc.sample_chain(5, q0, kernel=k, num_burnin_steps=2, trace_fn=None, seed=(9, 1))
  python = pg.mcmc.sample_chain(5, q0, kernel=k, num_burnin_steps=2, trace_fn=lambda s, kr: (),
                                seed=(9, 1)).all_states
  assert torch.equal(native, python)


def test_run_chain_continues_exactly(pg):
  """Two calls with first_step advanced equal one long call."""
  t, _ = _target(pg, 600, 8, precision='mixed')
  q0 = torch.from_numpy(_problems.init_state(32, 8, seed=6)).cuda()
  mk = lambda: pg.mcmc.DualAveragingStepSizeAdaptation(
      pg.mcmc.NoUTurnSampler(t, step_size=0.1, max_tree_depth=6), num_adaptation_steps=8)
  full = pg.mcmc.run_chain(mk(), 10, q0, seed=(1, 1))
  a = pg.mcmc.run_chain(mk(), 4, q0, seed=(1, 1))
  b = pg.mcmc.run_chain(mk(), 6, a.final_state, seed=(1, 1), first_step=4,
                        step_size=a.final_step_size, da_state=a.final_da_state)
  assert torch.equal(full.all_states, torch.cat([a.all_states, b.all_states]))
  assert torch.equal(full.trace['step_size'][-1], b.trace['step_size'][-1])


def test_hmc_logistic_posterior_matches_long_oracle_moments(pg):
  """The HMC workload shape (1000 x 25, 64 chains, eps 0.03, L 10) at reduced
  length: posterior means agree with a long FP64 oracle run within Monte
  Carlo standard error, R-hat < 1.01 on the engine's draws."""
  from oracle import mcmc as omcmc, philox, targets as otargets
  X, y, _ = _problems.logreg_data(1000, 25, seed=0)
  t = pg.LogisticRegression(X, y)
  q0 = torch.from_numpy(_problems.init_state(64, 25, seed=0)).cuda()
  k = pg.mcmc.HamiltonianMonteCarlo(t, step_size=0.03, num_leapfrog_steps=10)
  run = pg.mcmc.run_chain(k, 600, q0, num_burnin_steps=300, seed=(11, 0))
  d = run.all_states.cpu().numpy()                      # [600, 64, 25]
  rhat = diagnostics.potential_scale_reduction(d, split_chains=True)
  assert np.all(rhat < 1.01), rhat.max()
  # Monte Carlo standard errors from the spread of independent chain means
  # (no autocorrelation estimate needed: HMC here is strongly antithetic).
  cm = d.mean(0)                                        # [64, 25]
  mean = cm.mean(0)
  se_e = cm.std(0, ddof=1) / np.sqrt(cm.shape[0])
  # FP64 oracle reference run (independent draws), 128 chains.
  o = otargets.LogisticRegression(X, y)
  x = _problems.init_state(128, 25, seed=1).astype(np.float64)
  lp, g = o(x)
  ref = []
  for s in range(500):
    r = omcmc.hmc_one_step(o, x, lp, g, 0.03, 10, philox.PhiloxDraws((77, s)))
    x, lp, g = r.next_state, r.target_log_prob, r.grads_target_log_prob
    if s >= 250:
      ref.append(x)
  ref = np.stack(ref)
  rcm = ref.mean(0)                                     # [128, 25]
  ref_mean = rcm.mean(0)
  se_r = rcm.std(0, ddof=1) / np.sqrt(rcm.shape[0])
  z = np.abs(mean - ref_mean) / np.sqrt(se_e ** 2 + se_r ** 2)
  assert np.all(z < 4.5), z.max()
