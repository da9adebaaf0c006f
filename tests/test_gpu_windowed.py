"""windowed_adaptive_nuts (experimental/mcmc/windowed_sampling.py:603) on a
Gaussian whose scales span two orders of magnitude along the axes: the
diagonal mass matrix the slow windows estimate must approach the true
variances, adaptation must be flagged in the trace, and the draws after
adaptation must have the target's moments (within 5 Monte Carlo standard
errors, ESS summed over chains as in mcmc/nuts_test.py:398-399)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')


def test_windowed_adaptive_nuts_learns_the_diagonal_metric():
  if not torch.cuda.is_available():
    pytest.skip('no CUDA device')
  import probability_gb300 as pg
  from probability_gb300.experimental import mcmc as emcmc
  scales = np.array([0.1, 1.0, 3.0, 10.0])
  loc = np.array([1.0, -1.0, 0.0, 2.0])
  target = pg.MultivariateNormalTriL(loc, np.diag(scales))
  draws, trace, fkr = emcmc.windowed_adaptive_nuts(
      400, target, n_chains=64, num_adaptation_steps=500, seed=(11, 12),
      return_final_kernel_results=True)
  assert draws.shape == (400, 64, 4)
  precision = fkr.inner_results.inner_results.inner_results.momentum_distribution.precision_diag
  np.testing.assert_allclose(precision.cpu().numpy(), scales ** 2, rtol=0.3)
  assert not bool(trace['tune'][-1]) and trace['step_size'].shape[0] == 400
  x = draws.to(torch.float64)
  ess = pg.mcmc.effective_sample_size(x).sum(0).cpu().numpy()      # [4], over chains
  mean = x.mean((0, 1)).cpu().numpy()
  sd = x.std((0, 1)).cpu().numpy()
  assert np.all(np.abs(mean - loc) <= 5 * sd / np.sqrt(ess))
  np.testing.assert_allclose(sd, scales, rtol=0.1)
  assert float(pg.mcmc.potential_scale_reduction(x, split_chains=True).max()) < 1.02
