"""The package's torch ESS / R-hat / streaming statistics (used by bench.py for
min-ESS/s and by the job server) against the NumPy oracle of
mcmc/diagnostic.py:203-568 and experimental/stats/sample_stats.py
RunningVariance, on CPU tensors."""
import numpy as np
import pytest
import torch

from oracle import diagnostics
from probability_gb300.experimental import stats
from probability_gb300.mcmc import diagnostic


def _ar1(n, chains, dims, rho, seed):
  """AR(1) draws [n, chains, dims] with per-dimension correlation rho and
  per-chain offsets (so R-hat sees between-chain variance)."""
  rng = np.random.default_rng(seed)
  x = np.empty((n, chains, dims))
  x[0] = rng.normal(size=(chains, dims))
  for t in range(1, n):
    x[t] = rho * x[t - 1] + np.sqrt(1.0 - rho * rho) * rng.normal(size=(chains, dims))
  return x + 0.3 * rng.normal(size=(1, chains, 1))


@pytest.mark.parametrize('rho', [0.0, 0.6, 0.95, -0.4])
# filter_threshold=None (no truncation) is left out: mean-centred sample
# autocovariances sum to zero over all lags, so its denominator is zero up to
# roundoff and the value is undefined.
@pytest.mark.parametrize('kw', [{}, {'filter_threshold': 0.2},
                                {'filter_beyond_positive_pairs': True},
                                {'cross_chain_dims': 1},
                                {'cross_chain_dims': 1, 'filter_beyond_positive_pairs': True}])
def test_ess_matches_oracle(rho, kw):
  x = _ar1(301, 8, 3, rho, seed=int(100 * abs(rho)) + len(kw))
  got = diagnostic.effective_sample_size(torch.from_numpy(x), **kw).numpy()
  want = diagnostics.effective_sample_size(x, **kw)
  np.testing.assert_allclose(got, want, rtol=1e-9, atol=1e-9)


@pytest.mark.parametrize('lag', [1, 10, 64])
@pytest.mark.parametrize('kw', [{}, {'filter_beyond_positive_pairs': True},
                                {'cross_chain_dims': 1}])
def test_ess_filter_beyond_lag_matches_oracle(lag, kw):
  x = _ar1(257, 6, 3, 0.7, seed=lag)
  got = diagnostic.effective_sample_size(torch.from_numpy(x), filter_beyond_lag=lag,
                                         **kw).numpy()
  want = diagnostics.effective_sample_size(x, filter_beyond_lag=lag, **kw)
  np.testing.assert_allclose(got, want, rtol=1e-9, atol=1e-9)


@pytest.mark.parametrize('split', [False, True])
@pytest.mark.parametrize('n', [200, 201])
def test_rhat_matches_oracle(split, n):
  x = _ar1(n, 6, 4, 0.5, seed=n)
  got = diagnostic.potential_scale_reduction(torch.from_numpy(x), split_chains=split).numpy()
  want = diagnostics.potential_scale_reduction(x, split_chains=split)
  np.testing.assert_allclose(got, want, rtol=1e-12)


def test_running_variance_batches_equal_full_pass():
  rng = np.random.default_rng(7)
  x = rng.normal(size=(97, 5, 3)) * 3.0 + 2.0
  rv = stats.RunningVariance.from_shape((5, 3))
  for lo, hi in [(0, 1), (1, 40), (40, 41), (41, 97)]:
    rv = rv.update(torch.from_numpy(x[lo:hi]), axis=0)
  np.testing.assert_allclose(rv.mean.numpy(), x.mean(0), rtol=1e-12)
  np.testing.assert_allclose(rv.variance().numpy(), x.var(0), rtol=1e-10)
  np.testing.assert_allclose(rv.variance(ddof=1).numpy(), x.var(0, ddof=1), rtol=1e-10)
  # single samples (axis=None) give the same statistics
  rv1 = stats.RunningVariance.from_shape((5, 3))
  for t in range(x.shape[0]):
    rv1 = rv1.update(torch.from_numpy(x[t]))
  np.testing.assert_allclose(rv1.variance().numpy(), x.var(0), rtol=1e-10)


def test_running_rhat_from_moments_matches_oracle():
  """R-hat from per-chain running moments (what the device Welford update
  keeps) equals the batch formula over the stored draws."""
  x = _ar1(150, 8, 5, 0.3, seed=11)
  mean = torch.from_numpy(x.mean(0))
  m2 = torch.from_numpy(((x - x.mean(0, keepdims=True)) ** 2).sum(0))
  r = stats.RunningPotentialScaleReduction.from_moments(mean, m2, x.shape[0])
  np.testing.assert_allclose(r.potential_scale_reduction().numpy(),
                             diagnostics.potential_scale_reduction(x), rtol=1e-10)
