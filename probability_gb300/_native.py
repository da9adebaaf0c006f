"""ctypes binding of the engine's C ABI (include/gb300_mcmc.h).

The shared library is built in-tree by ``python -m probability_gb300.build``
(``__graft_entry__.build()`` does the same).  Nothing here has a CPU
fallback: if the library or a GPU is missing, the first call raises.
"""
import ctypes
import os
import threading

import torch

_LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'lib',
                         'libgb300mcmc.so')
_lib = None
_lock = threading.Lock()

GBM_OK = 0
GBM_EINVAL = 22
GBM_ENOMEM = 12
GBM_ENOTSUP = 95
GBM_ETIMEDOUT = 110
GBM_ECUDA = 1000
DTYPE_F32 = 0
DTYPE_BF16 = 1
PRECISION_F32 = 0
PRECISION_MIXED = 1

P = ctypes.c_void_p
I32 = ctypes.c_int32
I64 = ctypes.c_int64
F32 = ctypes.c_float
F64 = ctypes.c_double
U32P = ctypes.POINTER(ctypes.c_uint32)

_SIGNATURES = {
    'gbm_version': ([], ctypes.c_int),
    'gbm_last_error': ([], ctypes.c_char_p),
    'gbm_context_create': ([ctypes.c_int, P, ctypes.POINTER(P)], ctypes.c_int),
    'gbm_context_destroy': ([P], ctypes.c_int),
    'gbm_context_synchronize': ([P], ctypes.c_int),
    'gbm_target_logistic_regression': (
        [P, P, ctypes.c_int, I64, I64, P, F32, ctypes.c_int, ctypes.POINTER(P)], ctypes.c_int),
    'gbm_target_destroy': ([P], ctypes.c_int),
    'gbm_target_transformed': ([P, P, ctypes.POINTER(P)], ctypes.c_int),
    'gbm_target_mvn': ([P, P, P, I64, F64, ctypes.POINTER(P)], ctypes.c_int),
    'gbm_target_hierarchical_normal': ([P, P, P, I64, F32, F32, ctypes.POINTER(P)],
                                       ctypes.c_int),
    'gbm_target_dim': ([P, ctypes.POINTER(I64)], ctypes.c_int),
    'gbm_target_log_prob_and_grad': ([P, P, I64, P, P], ctypes.c_int),
    'gbm_target_cost': ([P, I64, ctypes.POINTER(F64), ctypes.POINTER(F64)], ctypes.c_int),
    'gbm_hmc_create': ([P, I64, ctypes.POINTER(P)], ctypes.c_int),
    'gbm_hmc_destroy': ([P], ctypes.c_int),
    'gbm_hmc_one_step': ([P, I64, P, P, P, P, ctypes.c_int, I32, U32P] + [P] * 11, ctypes.c_int),
    'gbm_nuts_create': ([P, I64, I32, F64, I32, ctypes.POINTER(P)], ctypes.c_int),
    'gbm_nuts_destroy': ([P], ctypes.c_int),
    'gbm_nuts_one_step': ([P, I64, P, P, P, P, ctypes.c_int, U32P] + [P] * 10, ctypes.c_int),
    'gbm_nuts_last_leaf_iterations': ([P, ctypes.POINTER(I64)], ctypes.c_int),
    'gbm_nuts_run_free': ([P, I64, P, P, P, P, ctypes.c_int, U32P, I64, I32, I64] + [P] * 7 +
                          [ctypes.POINTER(I64)], ctypes.c_int),
    'gbm_nuts_set_profiling': ([P, ctypes.c_int], ctypes.c_int),
    'gbm_nuts_set_graphs': ([P, ctypes.c_int], ctypes.c_int),
    'gbm_nuts_set_free_running': ([P, ctypes.c_int], ctypes.c_int),
    'gbm_moments_update': ([P, P, I64, I64, P, P], ctypes.c_int),
    'gbm_autocov_update': ([P, P, I64, I64, I32, P, P, P, P, P], ctypes.c_int),
    'gbm_nuts_set_inverse_mass': ([P, P, ctypes.c_int], ctypes.c_int),
    'gbm_nuts_read_profile': ([P, ctypes.POINTER(F64), ctypes.POINTER(I64),
                               ctypes.POINTER(I64)], ctypes.c_int),
    'gbm_dual_averaging_update': (
        [P, I64, P, ctypes.c_int, I32, F64, P, F64, F64, F64, P, P], ctypes.c_int),
    'gbm_dual_averaging_update_reduced': (
        [P, I64, P, I32, F64, P, F64, F64, F64, P, P], ctypes.c_int),
    'gbm_metropolis_hastings_step': ([P, I64, I64, U32P] + [P] * 8, ctypes.c_int),
    'gbm_step_key': ([U32P, ctypes.c_uint64, U32P], ctypes.c_int),
    'gbm_nuts_sample_chain': ([P, I64, P, P, P, P, ctypes.c_int, U32P, I64, I64, I64, I64, I32,
                               F64, F64, F64, F64] + [P] * 8, ctypes.c_int),
    'gbm_hmc_sample_chain': ([P, I64, P, P, P, P, ctypes.c_int, I32, U32P, I64, I64, I64, I64,
                              I32, F64, F64, F64, F64] + [P] * 6, ctypes.c_int),
    'gbm_logreg_log_prob_and_grad_noalloc': ([P, I64, I64, P, F32, P, I64, P, P, P],
                                             ctypes.c_int),
}


def lib():
  """Load (once) and return the engine library; raise if it is not built."""
  global _lib
  if _lib is not None:
    return _lib
  with _lock:
    if _lib is None:
      if not os.path.exists(_LIB_PATH):
        raise RuntimeError(
            'gb300 MCMC engine library not found at %s; build it with '
            '`python -m probability_gb300.build`' % _LIB_PATH)
      L = ctypes.CDLL(_LIB_PATH)
      for name, (args, res) in _SIGNATURES.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
      _lib = L
  return _lib


def library_path():
  return _LIB_PATH


def exported_symbols():
  return sorted(_SIGNATURES)


def check(status, what=''):
  if status == GBM_OK:
    return
  msg = lib().gbm_last_error().decode(errors='replace')
  text = '%s: %s' % (what, msg) if what else msg
  if status == GBM_EINVAL:
    raise ValueError(text)
  if status == GBM_ENOMEM:
    raise MemoryError(text)
  if status == GBM_ENOTSUP:
    raise NotImplementedError(text)
  if status == GBM_ETIMEDOUT:
    raise TimeoutError(text)
  raise RuntimeError(text)


def ptr(t):
  """Device pointer of a tensor (None -> NULL)."""
  if t is None:
    return None
  return ctypes.c_void_p(t.data_ptr())


def seed_words(seed):
  arr = (ctypes.c_uint32 * 2)(int(seed[0]) & 0xFFFFFFFF, int(seed[1]) & 0xFFFFFFFF)
  return arr


class Context:
  """One engine context per (device, stream); streams are torch's."""
  _cache = {}

  def __init__(self, device, stream):
    self.device = device
    self.stream = stream
    h = P()
    check(lib().gbm_context_create(device, P(stream.cuda_stream), ctypes.byref(h)),
          'gbm_context_create')
    self.handle = h

  @classmethod
  def current(cls, device=None):
    if not torch.cuda.is_available():
      raise RuntimeError('the gb300 MCMC engine needs a CUDA device; none is available')
    dev = torch.device('cuda', torch.cuda.current_device() if device is None else device)
    stream = torch.cuda.current_stream(dev)
    key = (dev.index, stream.cuda_stream)
    ctx = cls._cache.get(key)
    if ctx is None:
      ctx = cls(dev.index, stream)
      cls._cache[key] = ctx
    return ctx

  def synchronize(self):
    check(lib().gbm_context_synchronize(self.handle), 'gbm_context_synchronize')
