"""Batches larger than one launch of the logistic-regression kernels.

Each kernel launch covers at most (grid x chain tile) chains: one work item
per CTA (or CTA pair).  On a 152-SM GB300 that is 19,456 chains for the
FP32 kernel (2 x SMs x 64) and the chain-major tensor-core kernel
(SMs x 128, D <= 128), 9,728 for the row-major kernel (SMs x 64,
128 < D <= 256) and (resident pairs x 64) for the pair-cluster kernel
(256 < D <= 512).  Larger batches run as consecutive chunks; every chain
must come out equal to the FP64 oracle at the tolerances of the
single-launch parity tests (FP32: log-density rtol 2e-6, gradient rtol
1e-4 + 2e-5 max|grad|; mixed on BF16 data: log-density rtol 1e-5,
gradient 1e-3 max|grad|; mixed on FP32 data: gradient 2e-3 max|grad|).
The math is the inference_gym logistic-regression target
(spinoffs/inference_gym/inference_gym/targets/logistic_regression.py:92-103).
"""
import numpy as np
import pytest

from oracle import targets as otargets
from tests import _problems

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')

CHAINS = 25000


@pytest.fixture(scope='module')
def pg():
  if not torch.cuda.is_available():
    pytest.skip('no CUDA device')
  import probability_gb300 as pg
  return pg


@pytest.mark.parametrize('n,d,precision,bf16', [
    (2000, 25, 'fp32', False),
    (2000, 25, 'mixed', False),     # chain-major kernel, FP32 data (hi + lo)
    (2000, 100, 'mixed', True),     # chain-major kernel, BF16 data
    (2000, 200, 'mixed', True),     # row-major kernel
    (1000, 300, 'mixed', True),     # pair-cluster kernel
])
def test_more_chains_than_one_launch_covers(pg, n, d, precision, bf16):
  X, y, _ = _problems.logreg_data(n, d, seed=d + 3, scale=d ** -0.5)
  if bf16:
    Xb = torch.from_numpy(X).to(torch.bfloat16)
    t = pg.LogisticRegression(Xb, y, precision=precision)
    o = otargets.LogisticRegression(Xb.to(torch.float32).numpy(), y)
  else:
    t = pg.LogisticRegression(X, y, precision=precision)
    o = otargets.LogisticRegression(X, y)
  q = (np.random.default_rng(d).normal(size=(CHAINS, d)) * 0.5).astype(np.float32)
  lp, g = t.log_prob_and_grad(torch.from_numpy(q).cuda())
  lp, g = lp.cpu().numpy(), g.cpu().numpy()
  lp_o, g_o = o(q)
  scale = np.abs(g_o).max()
  if precision == 'fp32':
    np.testing.assert_allclose(lp, lp_o, rtol=2e-6, atol=1e-4)
    np.testing.assert_allclose(g, g_o, rtol=1e-4, atol=2e-5 * scale)
  else:
    np.testing.assert_allclose(lp, lp_o, rtol=1e-5, atol=1e-2)
    np.testing.assert_allclose(g, g_o, rtol=0, atol=(1e-3 if bf16 else 2e-3) * scale)
  # The last chunk's chains are not a copy of the first chunk's.
  assert not np.allclose(g[-100:], g[:100])
