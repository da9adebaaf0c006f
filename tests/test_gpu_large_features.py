"""Logistic regression above the fused kernels' feature limits (FP32 above
256 features, mixed precision above 512 -- the serving workload draws up to
1000): library GEMMs with FP32 accumulation and the library's own element-wise
kernels, against the FP64 oracle of the inference_gym target
(spinoffs/inference_gym/inference_gym/targets/logistic_regression.py:92-103).

Tolerances as the fused kernels': FP32 log-density rtol 2e-6, gradient rtol
1e-4 + 2e-5 max|grad|; mixed (BF16 hi/lo residual correction in both
contractions) log-density rtol 1e-5, gradient 2e-5 max|grad|, on X rounded
to BF16 (BF16 data) or on the FP32 data itself.
"""
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


@pytest.mark.parametrize('n,d,c', [(3000, 300, 70), (1500, 700, 129), (777, 257, 3),
                                   (9000, 400, 50)])
def test_fp32_above_256_features(pg, n, d, c):
  X, y, _ = _problems.logreg_data(n, d, seed=d, scale=d ** -0.5)
  t = pg.LogisticRegression(X, y, precision='fp32')
  q = (np.random.default_rng(c).normal(size=(c, d)) * 0.5).astype(np.float32)
  lp, g = t.log_prob_and_grad(torch.from_numpy(q).cuda())
  lp_o, g_o = otargets.LogisticRegression(X, y)(q)
  np.testing.assert_allclose(lp.cpu().numpy(), lp_o, rtol=2e-6, atol=1e-4)
  scale = np.abs(g_o).max()
  np.testing.assert_allclose(g.cpu().numpy(), g_o, rtol=1e-4, atol=2e-5 * scale)


@pytest.mark.parametrize('n,d,c,bf16', [(3000, 600, 64, True), (2000, 1000, 200, True),
                                        (1000, 513, 1, True), (2500, 800, 33, False),
                                        (9000, 600, 33, True), (8192, 700, 40, False)])
def test_mixed_above_512_features(pg, n, d, c, bf16):
  X, y, _ = _problems.logreg_data(n, d, seed=d + 1, scale=d ** -0.5)
  if bf16:
    Xb = torch.from_numpy(X).to(torch.bfloat16)
    t = pg.LogisticRegression(Xb, y, precision='mixed')
    o = otargets.LogisticRegression(Xb.to(torch.float32).numpy(), y)
  else:
    t = pg.LogisticRegression(X, y, precision='mixed')
    o = otargets.LogisticRegression(X, y)
  q = (np.random.default_rng(c).normal(size=(c, d)) * 0.5).astype(np.float32)
  lp, g = t.log_prob_and_grad(torch.from_numpy(q).cuda())
  lp_o, g_o = o(q)
  np.testing.assert_allclose(lp.cpu().numpy(), lp_o, rtol=1e-5, atol=1e-2)
  scale = np.abs(g_o).max()
  np.testing.assert_allclose(g.cpu().numpy(), g_o, rtol=0, atol=2e-5 * scale)


def test_nuts_transition_at_1000_features_tracks_oracle(pg):
  X, y, _ = _problems.logreg_data(1500, 1000, seed=5, scale=1000 ** -0.5)
  Xr = torch.from_numpy(X).to(torch.bfloat16)
  t = pg.LogisticRegression(Xr, y, precision='mixed')
  o = otargets.LogisticRegression(Xr.to(torch.float32).numpy(), y)
  C, D = 16, 1000
  q = torch.from_numpy(_problems.init_state(C, D, seed=6, scale=0.05)).cuda()
  k = pg.mcmc.NoUTurnSampler(t, step_size=0.01, max_tree_depth=5)
  kr = k.bootstrap_results(q)
  q1, kr1 = k.one_step(q, kr, seed=(2, 9))
  r = omcmc.nuts_one_step(o, q.cpu().numpy(), kr.target_log_prob.cpu().numpy(),
                          kr.grads_target_log_prob.cpu().numpy(), np.float32(0.01),
                          philox.PhiloxDraws((2, 9)), 5)
  same = kr1.leapfrogs_taken.cpu().numpy() == r.leapfrogs_taken
  assert same.mean() >= 0.9
  np.testing.assert_allclose(q1.cpu().numpy()[same], r.next_state[same], rtol=1e-5, atol=1e-5)
