"""Streaming diagnostics on the device (gbm_moments_update,
RunningPotentialScaleReduction; the job server's optional moment outputs):
equal to the stored-draw computations of diagnostic.py:476-568."""
import numpy as np
import pytest

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
  ref = pg.mcmc.potential_scale_reduction(draws.to(torch.float64), split_chains=False)
  np.testing.assert_allclose(r.potential_scale_reduction().cpu().numpy(), ref.cpu().numpy(),
                             rtol=1e-9)
  np.testing.assert_allclose(r.mean.cpu().numpy(), draws.double().mean(0).cpu().numpy(),
                             rtol=1e-12, atol=1e-12)


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
