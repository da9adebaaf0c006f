"""The allocation-free logistic-regression entry point.

gbm_logreg_log_prob_and_grad_noalloc exists for callers that cannot
allocate device memory (a framework's custom-call slot that only hands over
its own buffers, or a serving loop that must not synchronise the device in
cudaMalloc/cudaFree).  Its scratch lives in a fixed device array inside the
library, shared by every call.  This file is collected last so a run that
stops at the first failure has run everything else first; it also passes
alone in a fresh process.

Checked: two calls in a row (different batch sizes and states, so the second
call runs over the first call's leftover scratch) match the allocating entry
point gbm_target_log_prob_and_grad within the parity tests' tolerances
(log-density rtol 2e-6 / atol 1e-4; gradient rtol 1e-4, atol 2e-5 x max
|grad|), and oversize requests are rejected with GBM_EINVAL.
"""
import ctypes

import numpy as np
import pytest

from tests import _problems

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')


def _noalloc(lib, _native, X, y, q, prior_scale=1.0):
  C, D = q.shape
  lp = torch.empty(C, dtype=torch.float64, device='cuda')
  g = torch.empty((C, D), dtype=torch.float32, device='cuda')
  st = lib.gbm_logreg_log_prob_and_grad_noalloc(
      _native.ptr(X), X.shape[0], X.shape[1], _native.ptr(y), prior_scale, _native.ptr(q), C,
      _native.ptr(lp), _native.ptr(g), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
  return st, lp, g


def test_noalloc_matches_allocating_entry_point_twice():
  if not torch.cuda.is_available():
    pytest.skip('no CUDA device')
  import probability_gb300 as pg
  from probability_gb300 import _native
  lib = _native.lib()
  Xn, yn, _ = _problems.logreg_data(3000, 100, seed=21, scale=0.1)
  X = torch.from_numpy(Xn).cuda()
  y = torch.from_numpy(yn).cuda()
  target = pg.LogisticRegression(Xn, yn)
  rng = np.random.default_rng(5)
  for chains in (300, 77):                      # two calls in a row
    q = torch.from_numpy((rng.normal(size=(chains, 100)) * 0.2).astype(np.float32)).cuda()
    st, lp, g = _noalloc(lib, _native, X, y, q)
    assert st == 0, lib.gbm_last_error()
    torch.cuda.synchronize()
    lp_ref, g_ref = target.log_prob_and_grad(q)
    np.testing.assert_allclose(lp.cpu().numpy(), lp_ref.cpu().numpy(), rtol=2e-6, atol=1e-4)
    scale = float(g_ref.abs().max())
    np.testing.assert_allclose(g.cpu().numpy(), g_ref.cpu().numpy(), rtol=1e-4,
                               atol=2e-5 * scale)


def test_noalloc_rejects_sizes_beyond_its_scratch():
  if not torch.cuda.is_available():
    pytest.skip('no CUDA device')
  from probability_gb300 import _native
  lib = _native.lib()
  Xn, yn, _ = _problems.logreg_data(100, 256, seed=3)
  X = torch.from_numpy(Xn).cuda()
  y = torch.from_numpy(yn).cuda()
  q = torch.zeros((9000, 256), dtype=torch.float32, device='cuda')
  st, _, _ = _noalloc(lib, _native, X, y, q)
  assert st == _native.GBM_EINVAL
  assert b'exceed' in lib.gbm_last_error()
  Xw = torch.zeros((10, 300), dtype=torch.float32, device='cuda')
  st, _, _ = _noalloc(lib, _native, Xw, y[:10], torch.zeros((2, 300), device='cuda'))
  assert st == _native.GBM_EINVAL
