"""Mixed-precision (tcgen05, BF16 operands with hi/lo residual correction,
FP32 accumulation) logistic-regression target against the FP64 oracle.

X is BF16 in this path; the oracle is evaluated on the same BF16-rounded X,
so the only error is the engine's arithmetic.  Stated tolerances:
log-density rtol 1e-5 (+1e-2 absolute); gradient, absolute, relative to
max|grad|: 2e-5 up to 128 features (the chain-major kernel splits the
residuals R into BF16 hi + lo and, for FP32 data, adds X_lo, so the gradient
contraction is residual-corrected too), 1e-3 above 128 features (R enters
the contraction as BF16 there).
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


def _bf16_round(x):
  return torch.from_numpy(x).to(torch.bfloat16).to(torch.float32).numpy()


@pytest.mark.parametrize('n,d,c', [(1000, 25, 64), (5000, 100, 300), (3000, 200, 70),
                                   (130, 7, 1), (4096, 128, 128), (777, 250, 129),
                                   # 256 < D <= 512: the pair-cluster kernel
                                   (3000, 300, 70), (777, 512, 129), (2000, 257, 64),
                                   (5000, 400, 300), (129, 511, 1)])
def test_mixed_log_prob_and_grad_vs_fp64(pg, n, d, c):
  X, y, _ = _problems.logreg_data(n, d, seed=n + 7 * d, scale=1.0 / np.sqrt(d))
  Xb = torch.from_numpy(X).to(torch.bfloat16)
  t = pg.LogisticRegression(Xb, y, precision='mixed')
  o = otargets.LogisticRegression(Xb.to(torch.float32).numpy(), y)
  q = (np.random.default_rng(c).normal(size=(c, d)) * 0.5).astype(np.float32)
  lp, g = t.log_prob_and_grad(torch.from_numpy(q).cuda())
  lp_o, g_o = o(q)
  np.testing.assert_allclose(lp.cpu().numpy(), lp_o, rtol=1e-5, atol=1e-2)
  scale = np.abs(g_o).max()
  np.testing.assert_allclose(g.cpu().numpy(), g_o, rtol=0, atol=_grad_tol(d) * scale)


def _grad_tol(d):
  return 2e-5 if d <= 128 else 1e-3


@pytest.mark.parametrize('n,d,c', [(5000, 100, 300), (1000, 25, 64), (257, 128, 129)])
def test_mixed_on_fp32_data_keeps_fp32_fidelity(pg, n, d, c):
  """FP32 X (up to 128 features) is kept as BF16 hi + lo; the log-density is
  then that of the FP32 data, not of X rounded to BF16."""
  X, y, _ = _problems.logreg_data(n, d, seed=2 * n + d, scale=1.0 / np.sqrt(d))
  t = pg.LogisticRegression(X, y, precision='mixed')
  o = otargets.LogisticRegression(X, y)
  q = (np.random.default_rng(c).normal(size=(c, d)) * 0.5).astype(np.float32)
  lp, g = t.log_prob_and_grad(torch.from_numpy(q).cuda())
  lp_o, g_o = o(q)
  np.testing.assert_allclose(lp.cpu().numpy(), lp_o, rtol=1e-5, atol=1e-2)
  scale = np.abs(g_o).max()
  np.testing.assert_allclose(g.cpu().numpy(), g_o, rtol=0, atol=2e-5 * scale)


def test_mixed_at_full_1e5x100_shape_vs_fp64():
  """The 1e5 x 100, 1024-chain shape of the NUTS workload (FP32 data, column
  0 = 1, other columns N(0, 1)/10), at states drawn around the posterior
  mode (its Laplace approximation), against the FP64 oracle.  The gradient
  bound here is 2e-4 x max|grad|: with R and X split into BF16 hi + lo the
  remaining error is the tensor cores' FP32 accumulation of G over the
  ~5,000 rows of each row split (about 7e-5 x max|grad| measured), which
  grows with the rows a CTA sums."""
  if not torch.cuda.is_available():
    pytest.skip('no CUDA device')
  import probability_gb300 as pg
  X, y, _ = _problems.logreg_data(100000, 100, seed=1, scale=0.1)
  mode, H = _problems.laplace(X, y)
  L = np.linalg.cholesky(np.linalg.inv(H))
  q = (mode + np.random.default_rng(3).standard_normal((1024, 100)) @ L.T).astype(np.float32)
  t = pg.LogisticRegression(X, y, precision='mixed')
  lp, g = t.log_prob_and_grad(torch.from_numpy(q).cuda())
  lp, g = lp.cpu().numpy(), g.cpu().numpy()
  o = otargets.LogisticRegression(X, y)
  for c0 in range(0, 1024, 128):
    lp_o, g_o = o(q[c0:c0 + 128])
    np.testing.assert_allclose(lp[c0:c0 + 128], lp_o, rtol=1e-5, atol=1e-2)
    scale = np.abs(g_o).max()
    np.testing.assert_allclose(g[c0:c0 + 128], g_o, rtol=0, atol=2e-4 * scale)


def test_mixed_matches_fp32_target_on_same_data(pg):
  X, y, _ = _problems.logreg_data(3000, 100, seed=3, scale=0.1)
  Xr = _bf16_round(X)
  tm = pg.LogisticRegression(torch.from_numpy(Xr).to(torch.bfloat16), y, precision='mixed')
  tf = pg.LogisticRegression(Xr, y, precision='fp32')
  q = torch.from_numpy((np.random.default_rng(0).normal(size=(256, 100)) * 0.3)
                       .astype(np.float32)).cuda()
  lm, gm = tm.log_prob_and_grad(q)
  lf, gf = tf.log_prob_and_grad(q)
  np.testing.assert_allclose(lm.cpu().numpy(), lf.cpu().numpy(), rtol=1e-5, atol=1e-2)
  np.testing.assert_allclose(gm.cpu().numpy(), gf.cpu().numpy(), rtol=0,
                             atol=2e-5 * float(gf.abs().max()))


def test_mixed_nuts_transition_tracks_oracle(pg):
  X, y, _ = _problems.logreg_data(2000, 25, seed=9, scale=0.5)
  Xr = _bf16_round(X)
  t = pg.LogisticRegression(torch.from_numpy(Xr).to(torch.bfloat16), y, precision='mixed')
  o = otargets.LogisticRegression(Xr, y)
  C, D = 64, 25
  q = torch.from_numpy(_problems.init_state(C, D, seed=4)).cuda()
  k = pg.mcmc.NoUTurnSampler(t, step_size=0.02, max_tree_depth=7)
  kr = k.bootstrap_results(q)
  q1, kr1 = k.one_step(q, kr, seed=(8, 8))
  r = omcmc.nuts_one_step(o, q.cpu().numpy(), kr.target_log_prob.cpu().numpy(),
                          kr.grads_target_log_prob.cpu().numpy(), np.float32(0.02),
                          philox.PhiloxDraws((8, 8)), 7)
  same = kr1.leapfrogs_taken.cpu().numpy() == r.leapfrogs_taken
  assert same.mean() >= 0.95
  # The FP32 criterion (1e-5 relative) on chains whose trajectories agree.
  np.testing.assert_allclose(q1.cpu().numpy()[same], r.next_state[same], rtol=1e-5, atol=1e-5)
