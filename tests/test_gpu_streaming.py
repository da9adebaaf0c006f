"""Streaming diagnostics on the device (gbm_moments_update,
RunningPotentialScaleReduction with and without split chains,
gbm_autocov_update / RunningEffectiveSampleSize; the job server's optional
moment outputs): equal to the NumPy oracle of diagnostic.py:203-568 on the
stored draws (R-hat rtol 1e-9; ESS rtol 1e-6, the running sums being float64
over float32 draws)."""
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


def test_running_rhat_equals_stored_draws(pg):
  from probability_gb300.experimental.stats import RunningPotentialScaleReduction
  g = torch.Generator(device='cuda')
  g.manual_seed(0)
  draws = torch.randn(50, 8, 5, device='cuda', generator=g) + \
      torch.linspace(0, 0.5, 8, device='cuda')[None, :, None]
  r = RunningPotentialScaleReduction((8, 5))
  for x in draws:
    r.update(x)
  ref = diagnostics.potential_scale_reduction(draws.double().cpu().numpy(), split_chains=False)
  np.testing.assert_allclose(r.potential_scale_reduction().cpu().numpy(), ref, rtol=1e-9)
  np.testing.assert_allclose(r.mean.cpu().numpy(), draws.double().mean(0).cpu().numpy(),
                             rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize('n', [50, 51])
def test_running_split_rhat_equals_oracle(pg, n):
  from probability_gb300.experimental.stats import RunningPotentialScaleReduction
  g = torch.Generator(device='cuda')
  g.manual_seed(n)
  # A drift within each chain, which split R-hat detects and plain R-hat
  # does not.
  draws = torch.randn(n, 8, 5, device='cuda', generator=g) + \
      torch.linspace(0, 2.0, n, device='cuda')[:, None, None]
  r = RunningPotentialScaleReduction((8, 5), split_chains=True, num_draws=n)
  for x in draws:
    r.update(x)
  ref = diagnostics.potential_scale_reduction(draws.double().cpu().numpy(), split_chains=True)
  got = r.potential_scale_reduction().cpu().numpy()
  np.testing.assert_allclose(got, ref, rtol=1e-9)
  assert got.min() > 1.1


@pytest.mark.parametrize('kw', [{}, {'filter_beyond_positive_pairs': True},
                                {'cross_chain_dims': 1},
                                {'cross_chain_dims': 1, 'filter_beyond_positive_pairs': True}])
def test_running_ess_equals_oracle_with_lag_truncation(pg, kw):
  from probability_gb300.experimental.stats import RunningEffectiveSampleSize
  rng = np.random.default_rng(len(kw))
  n, C, D, L = 300, 8, 3, 40
  x = np.empty((n, C, D))
  x[0] = rng.normal(size=(C, D))
  for t in range(1, n):                        # AR(1), correlation 0.8, offset mean
    x[t] = 0.8 * x[t - 1] + 0.6 * rng.normal(size=(C, D))
  x = (x + 5.0).astype(np.float32)
  r = RunningEffectiveSampleSize((C, D), max_lag=L)
  for t in range(n):
    r.update(torch.from_numpy(x[t]).cuda())
  want = diagnostics.effective_sample_size(x.astype(np.float64), filter_beyond_lag=L, **kw)
  got = r.effective_sample_size(**kw).cpu().numpy()
  np.testing.assert_allclose(got, want, rtol=1e-6)
  acov = diagnostics.auto_covariance(x.astype(np.float64), 0)[:L + 1]
  np.testing.assert_allclose(r.auto_covariance().cpu().numpy(), acov, rtol=1e-6, atol=1e-9)


def test_server_job_moments_match_its_draws(pg):
  from probability_gb300.experimental.stats import RunningPotentialScaleReduction
  from probability_gb300.serving import Server, DONE
  X, y, _ = _problems.logreg_data(2000, 10, seed=2, scale=0.3)
  srv = Server(workers=1, memory_budget_bytes=2**30)
  job = srv.submit_logistic_regression(
      X, y, _problems.init_state(16, 10, seed=1), 30, num_burnin_steps=5, step_size=0.05,
      num_adaptation_steps=5, seed=(4, 4), trace=('state', 'moments'))
  assert job.wait()['status'] == DONE
  st = job.states.double()
  np.testing.assert_allclose(job.moments_mean.cpu().numpy(), st.mean(0).cpu().numpy(),
                             rtol=1e-10, atol=1e-10)
  np.testing.assert_allclose(job.moments_m2.cpu().numpy(),
                             ((st - st.mean(0)) ** 2).sum(0).cpu().numpy(), rtol=1e-8, atol=1e-9)
  r = RunningPotentialScaleReduction.from_moments(job.moments_mean, job.moments_m2, 30)
  np.testing.assert_allclose(r.potential_scale_reduction().cpu().numpy(),
                             pg.mcmc.potential_scale_reduction(st).cpu().numpy(), rtol=1e-8)
  srv.close()
