"""The job server (gbm_server_*): results equal the single-sampler path
(run_chain with free-running draws, as the server runs its jobs), are
identical alone and in a concurrent mix, and admission respects the
device-memory budget."""
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


def _logreg_job(server, seed, n=3000, d=20, chains=32, results=12, precision='mixed'):
  X, y, _ = _problems.logreg_data(n, d, seed=seed, scale=1.0 / np.sqrt(d))
  q0 = _problems.init_state(chains, d, seed=seed)
  return server.submit_logistic_regression(
      X, y, q0, results, precision=precision, num_burnin_steps=5, step_size=0.1,
      max_tree_depth=8, num_adaptation_steps=10, target_accept_prob=0.8, seed=(seed, 1))


def test_server_job_equals_run_chain(pg):
  from probability_gb300.serving import Server, DONE
  srv = Server(workers=2, memory_budget_bytes=4 * 2**30)
  job = _logreg_job(srv, seed=3)
  assert job.wait()['status'] == DONE
  X, y, _ = _problems.logreg_data(3000, 20, seed=3, scale=1.0 / np.sqrt(20))
  t = pg.LogisticRegression(X, y, precision='mixed')
  k = pg.mcmc.DualAveragingStepSizeAdaptation(
      pg.mcmc.NoUTurnSampler(t, step_size=0.1, max_tree_depth=8), num_adaptation_steps=10,
      target_accept_prob=0.8)
  run = pg.mcmc.run_chain(k, 12, torch.from_numpy(_problems.init_state(32, 20, seed=3)).cuda(),
                          num_burnin_steps=5, seed=(3, 1), free_running_draws=True)
  assert torch.equal(job.states, run.all_states)
  assert torch.equal(job.leapfrogs_taken, run.trace['leapfrogs_taken'])
  srv.close()


def test_server_result_is_the_same_alone_and_in_the_mix(pg):
  from probability_gb300.serving import Server, DONE
  srv = Server(workers=6, memory_budget_bytes=8 * 2**30)
  alone = _logreg_job(srv, seed=5)
  alone.wait()
  rng = np.random.default_rng(0)
  others = []
  for i in range(3):
    others.append(_logreg_job(srv, seed=10 + i, n=5000 + 1000 * i, d=30 + 10 * i, chains=64))
  d = 40
  A = rng.normal(size=(d, d + 2)) / np.sqrt(d)
  L = np.linalg.cholesky(A @ A.T)
  others.append(srv.submit_mvn(np.zeros(d), L, rng.normal(size=(48, d)).astype(np.float32), 10,
                               step_size=0.05, max_tree_depth=8, num_adaptation_steps=5,
                               seed=(7, 7)))
  J = 16
  sig = rng.uniform(5, 20, J)
  yj = rng.normal(size=J) * 10
  others.append(srv.submit_hierarchical_normal(
      yj, sig, (rng.normal(size=(64, J + 2)) * 0.5).astype(np.float32), 10, step_size=0.2,
      max_tree_depth=8, num_adaptation_steps=5, seed=(8, 8)))
  mixed = _logreg_job(srv, seed=5)
  for j in others + [mixed]:
    assert j.wait()['status'] == DONE
  # Same bits: no state is shared between concurrently running jobs.
  assert torch.equal(alone.states, mixed.states)
  assert torch.equal(alone.log_accept_ratio, mixed.log_accept_ratio)
  infos = [j.info() for j in others + [mixed]]
  starts = sorted(i['start_s'] for i in infos)
  ends = sorted(i['end_s'] for i in infos)
  assert starts[-1] < ends[-1]
  # Jobs overlapped on the device: some job started before another finished.
  assert any(a['start_s'] < b['end_s'] and b['start_s'] < a['end_s']
             for ai, a in enumerate(infos) for b in infos[ai + 1:])
  srv.close()


def test_server_admission_respects_budget(pg):
  from probability_gb300.serving import Server, DONE
  one = _problems.logreg_data(3000, 20, seed=1)
  srv = Server(workers=4, memory_budget_bytes=1)
  with pytest.raises(MemoryError):
    _logreg_job(srv, seed=1)
  srv.close()
  # A budget that fits one job at a time serializes them.
  probe = Server(workers=1, memory_budget_bytes=4 * 2**30)
  j = _logreg_job(probe, seed=2)
  need = j.wait()['device_bytes']
  probe.close()
  srv = Server(workers=4, memory_budget_bytes=int(need * 1.5))
  jobs = [_logreg_job(srv, seed=20 + i) for i in range(3)]
  infos = [j.wait() for j in jobs]
  assert all(i['status'] == DONE for i in infos)
  for a, b in zip(infos, infos[1:]):
    assert b['start_s'] >= a['end_s'] - 1e-6
  srv.close()


@pytest.mark.parametrize('d,precision', [(300, 'fp32'), (600, 'mixed')])
def test_server_job_beyond_the_fused_kernels_feature_limits(pg, d, precision):
  """Above 256 (FP32) or 512 (mixed) features a job runs on the library-GEMM
  target and still equals the single-sampler path."""
  from probability_gb300.serving import Server, DONE
  srv = Server(workers=1, memory_budget_bytes=4 * 2**30)
  job = _logreg_job(srv, seed=7, n=1500, d=d, chains=24, results=4, precision=precision)
  assert job.wait()['status'] == DONE
  X, y, _ = _problems.logreg_data(1500, d, seed=7, scale=1.0 / np.sqrt(d))
  t = pg.LogisticRegression(X, y, precision=precision)
  k = pg.mcmc.DualAveragingStepSizeAdaptation(
      pg.mcmc.NoUTurnSampler(t, step_size=0.1, max_tree_depth=8), num_adaptation_steps=10,
      target_accept_prob=0.8)
  run = pg.mcmc.run_chain(k, 4, torch.from_numpy(_problems.init_state(24, d, seed=7)).cuda(),
                          num_burnin_steps=5, seed=(7, 1), free_running_draws=True)
  assert torch.equal(job.states, run.all_states)
  assert torch.equal(job.leapfrogs_taken, run.trace['leapfrogs_taken'])
  srv.close()


def test_server_rejects_bad_specs(pg):
  from probability_gb300.serving import Server
  srv = Server(workers=1, memory_budget_bytes=2**30)
  X, y, _ = _problems.logreg_data(100, 6, seed=1)
  with pytest.raises(ValueError):   # init_state width is not the feature count
    srv.submit_logistic_regression(X, y, np.zeros((4, 5), np.float32), 2)
  with pytest.raises(ValueError):   # the prior scale must be positive
    srv.submit_logistic_regression(X, y, np.zeros((4, 6), np.float32), 2, prior_scale=0.0)
  srv.close()
