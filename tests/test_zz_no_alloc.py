"""The allocation-free logistic-regression entry point.

gbm_logreg_log_prob_and_grad_noalloc exists for callers that cannot
allocate device memory (a framework's custom-call slot that only hands over
its own buffers, or a serving loop that must not synchronise the device in
cudaMalloc/cudaFree).  Its scratch lives in a fixed device array inside the
library, shared by every call.  This file is collected last so a run that
stops at the first failure has run everything else first; it also passes
alone in a fresh process.

Checked, for feature counts that exercise every register-tile width of the
kernel (7: 2 feature groups, 37: 4, 100: 8, 200: 16) and odd row strides
(the caller's X is read unpadded, row stride = features):
* two calls in a row (different batch sizes and states, so the second call
  runs over the first call's leftover scratch) match the allocating entry
  point gbm_target_log_prob_and_grad and the FP64 oracle within the parity
  tests' tolerances (log-density rtol 2e-6 / atol 1e-4; gradient rtol 1e-4,
  atol 2e-5 x max |grad|);
* a call at exactly the documented maximum chain count matches both too;
* one chain more, or more than 256 features, is rejected with GBM_EINVAL.
"""
import ctypes

import numpy as np
import pytest

from oracle import targets as otargets
from tests import _problems

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')

_SCRATCH = 8 << 20          # bytes of the library's fixed scratch array
_COUNT_BYTES = 256          # batch-size word at its start
_CT = 64                    # chains per work item


def _max_chains(features):
  """The documented limit: 64 * min(2 * SMs, floor((8 MiB - 256) /
  (64 * (8 + 4 * features))))."""
  sms = torch.cuda.get_device_properties(0).multi_processor_count
  fit = (_SCRATCH - _COUNT_BYTES) // (_CT * (8 + 4 * features))
  return _CT * min(2 * sms, fit)


def _noalloc(lib, _native, X, y, q, prior_scale=1.0):
  C, D = q.shape
  lp = torch.empty(C, dtype=torch.float64, device='cuda')
  g = torch.empty((C, D), dtype=torch.float32, device='cuda')
  st = lib.gbm_logreg_log_prob_and_grad_noalloc(
      _native.ptr(X), X.shape[0], X.shape[1], _native.ptr(y), prior_scale, _native.ptr(q), C,
      _native.ptr(lp), _native.ptr(g), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
  return st, lp, g


def _check(lp, g, lp_ref, g_ref):
  np.testing.assert_allclose(lp, lp_ref, rtol=2e-6, atol=1e-4)
  scale = float(np.abs(g_ref).max())
  np.testing.assert_allclose(g, g_ref, rtol=1e-4, atol=2e-5 * scale)


@pytest.fixture(scope='module')
def lib():
  if not torch.cuda.is_available():
    pytest.skip('no CUDA device')
  from probability_gb300 import _native
  return _native.lib()


@pytest.mark.parametrize('features', [7, 37, 100, 200])
def test_noalloc_matches_allocating_entry_point_and_oracle(lib, features):
  import probability_gb300 as pg
  from probability_gb300 import _native
  rows = 1000 + features          # ragged last row tile
  Xn, yn, _ = _problems.logreg_data(rows, features, seed=21 + features,
                                    scale=features ** -0.5)
  X = torch.from_numpy(Xn).cuda()
  y = torch.from_numpy(yn).cuda()
  target = pg.LogisticRegression(Xn, yn, precision='fp32')
  oracle = otargets.LogisticRegression(Xn, yn)
  rng = np.random.default_rng(5)
  limit = _max_chains(features)
  for chains in (300, 77, limit):  # calls in a row over the shared scratch
    qn = (rng.normal(size=(chains, features)) * 0.2).astype(np.float32)
    q = torch.from_numpy(qn).cuda()
    st, lp, g = _noalloc(lib, _native, X, y, q)
    assert st == 0, lib.gbm_last_error()
    torch.cuda.synchronize()
    lp_a, g_a = target.log_prob_and_grad(q)
    lp, g = lp.cpu().numpy(), g.cpu().numpy()
    _check(lp, g, lp_a.cpu().numpy(), g_a.cpu().numpy())
    lp_o, g_o = oracle(qn)
    _check(lp, g, lp_o, g_o)
  q = torch.zeros((limit + 1, features), dtype=torch.float32, device='cuda')
  st, _, _ = _noalloc(lib, _native, X, y, q)
  assert st == _native.GBM_EINVAL
  assert b'exceed' in lib.gbm_last_error()


def test_noalloc_rejects_sizes_beyond_its_scratch(lib):
  from probability_gb300 import _native
  Xn, yn, _ = _problems.logreg_data(100, 256, seed=3)
  X = torch.from_numpy(Xn).cuda()
  y = torch.from_numpy(yn).cuda()
  q = torch.zeros((_max_chains(256) + 1, 256), dtype=torch.float32, device='cuda')
  st, _, _ = _noalloc(lib, _native, X, y, q)
  assert st == _native.GBM_EINVAL
  assert b'exceed' in lib.gbm_last_error()
  Xw = torch.zeros((10, 300), dtype=torch.float32, device='cuda')
  st, _, _ = _noalloc(lib, _native, Xw, y[:10], torch.zeros((2, 300), device='cuda'))
  assert st == _native.GBM_EINVAL
