"""Long runs of DA(NUTS) on a logistic-regression posterior, in both
precisions: posterior means and variances must agree with the truth within
Monte Carlo standard error, and split R-hat must be below 1.01.

Modelled on the reference's testCorrelated2dNormalwithinMCError
(mcmc/nuts_test.py:358-425): independent replicas of 100 chains; per replica
and statistic the error |estimate - truth| is scaled by the Monte Carlo
standard error mean(std over draws) / sqrt(ESS summed over chains); a z-test
at p = 0.005 (two-sided 0.01) may fail for at most 5% of the tests.  The
truth is the FP64 importance-sampling estimate of tests/_problems.py (its
own standard error is added in quadrature).  The target is the
inference_gym logistic regression
(spinoffs/inference_gym/inference_gym/targets/logistic_regression.py:92-103);
'mixed' runs it with BF16 tensor-core contractions with residual correction.
"""
import math

import numpy as np
import pytest

from tests import _problems

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')

REPLICAS, CHAINS_PER_REPLICA, ADAPT, DRAWS = 10, 100, 300, 500


@pytest.fixture(scope='module')
def problem():
  if not torch.cuda.is_available():
    pytest.skip('no CUDA device')
  X, y, _ = _problems.logreg_data(2000, 4, seed=31, scale=0.5)
  return X, y, _problems.logreg_posterior_moments(X, y, n=200000, seed=7)


@pytest.mark.parametrize('precision', ['fp32', 'mixed'])
def test_posterior_moments_within_mc_error(problem, precision):
  import probability_gb300 as pg
  X, y, (mean_true, var_true, mean_se, var_se) = problem
  C = REPLICAS * CHAINS_PER_REPLICA
  t = pg.LogisticRegression(X, y, precision=precision)
  nuts = pg.mcmc.NoUTurnSampler(t, step_size=0.1, max_tree_depth=10)
  k = pg.mcmc.DualAveragingStepSizeAdaptation(nuts, num_adaptation_steps=ADAPT,
                                              target_accept_prob=0.8)
  q0 = torch.from_numpy(_problems.init_state(C, X.shape[1], seed=5)).cuda()
  run = pg.mcmc.run_chain(k, DRAWS, q0, num_burnin_steps=ADAPT, seed=(2024, 1))
  draws = run.all_states.to(torch.float64)                 # [draws, chains, D]
  rhat = pg.mcmc.potential_scale_reduction(draws, split_chains=True)
  assert float(rhat.max()) < 1.01
  mu = torch.as_tensor(mean_true, device=draws.device)
  samples = torch.cat([draws, (draws - mu) ** 2], -1)     # means, then variances
  truth = np.concatenate([mean_true, var_true])
  truth_se = np.concatenate([mean_se, var_se])
  ess = pg.mcmc.effective_sample_size(samples)             # [chains, 2D]
  failed, total = 0, 0
  for r in range(REPLICAS):
    sl = slice(r * CHAINS_PER_REPLICA, (r + 1) * CHAINS_PER_REPLICA)
    s = samples[:, sl]
    est = s.mean((0, 1)).cpu().numpy()
    mcse = (s.std(0).mean(0) / ess[sl].sum(0).sqrt()).cpu().numpy()
    z = np.abs(est - truth) / np.sqrt(mcse ** 2 + truth_se ** 2)
    p = 0.5 * np.array([math.erfc(v / math.sqrt(2.0)) for v in z])
    failed += int((p <= 0.005).sum())
    total += len(z)
  assert failed <= round(0.05 * total), (failed, total)
