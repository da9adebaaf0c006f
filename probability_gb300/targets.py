"""Built-in target families with fused log-density + gradient kernels.

The reference accepts any ``target_log_prob_fn`` and differentiates it with
autodiff (mcmc/internal/util.py:286-308).  This engine instead recognises
model-family descriptors and runs their hand-written fused kernels; each
descriptor is also a plain callable ``f(state) -> log_prob`` with the
reference's semantics.  Any other callable passed to a kernel raises
``NotImplementedError`` (there is no CPU or autodiff fallback).
"""
import ctypes

import numpy as np
import torch

from probability_gb300 import _native, _util


class Target:
  """Handle to a device-resident target; subclasses create ``_handle``."""

  _handle = None
  precision = 'fp32'

  @property
  def dim(self):
    d = ctypes.c_int64()
    _native.check(_native.lib().gbm_target_dim(self._handle, ctypes.byref(d)), 'gbm_target_dim')
    return int(d.value)

  def log_prob_and_grad(self, state):
    """Batched (log_prob float64 [C], grad float32 [C, D]) at ``state`` [C, D]."""
    q = _util.as_tensor(state, torch.float32)
    squeeze = q.dim() == 1
    q = q.reshape(-1, self.dim).contiguous()
    logp = torch.empty(q.shape[0], dtype=torch.float64, device=q.device)
    grad = torch.empty_like(q)
    _native.check(_native.lib().gbm_target_log_prob_and_grad(
        self._handle, _native.ptr(q), q.shape[0], _native.ptr(logp), _native.ptr(grad)),
        'gbm_target_log_prob_and_grad')
    if squeeze:
      return logp[0], grad[0]
    return logp, grad

  def __call__(self, state):
    return self.log_prob_and_grad(state)[0]

  def cost(self, chains):
    """(algorithmic flops, algorithmic HBM bytes) of one batched evaluation."""
    f, b = ctypes.c_double(), ctypes.c_double()
    _native.check(_native.lib().gbm_target_cost(self._handle, int(chains), ctypes.byref(f),
                                                ctypes.byref(b)), 'gbm_target_cost')
    return f.value, b.value

  def __del__(self):
    h = self._handle
    if h is not None and _native._lib is not None:
      try:
        _native.lib().gbm_target_destroy(h)
      except Exception:  # interpreter shutdown
        pass
      self._handle = None


class LogisticRegression(Target):
  """Bayesian logistic regression with an iid Normal(0, prior_scale) prior.

  ``features`` X is [N, D] (float32, or bfloat16 for the mixed-precision
  path) and already contains any intercept column; ``labels`` y is [N] in
  {0, 1}.  Matches the inference_gym logistic-regression target
  (spinoffs/inference_gym/inference_gym/targets/logistic_regression.py:88-103)
  with the intercept placed wherever the caller put it.

  precision: 'fp32' (CUDA-core FP32, the plain form) or 'mixed' (BF16 tensor
  cores with FP32 accumulation and hi/lo split residual correction).
  """

  def __init__(self, features, labels, prior_scale=1.0, precision='fp32'):
    if precision not in ('fp32', 'mixed'):
      raise ValueError("precision must be 'fp32' or 'mixed'")
    self.precision = precision
    X = _util.as_tensor(features)
    if X.dtype not in (torch.float32, torch.bfloat16):
      X = X.to(torch.float32)
    if precision == 'fp32' and X.dtype != torch.float32:
      X = X.to(torch.float32)
    if X.dim() != 2:
      raise ValueError('features must be [num_rows, num_features]')
    y = _util.as_tensor(labels, torch.float32).reshape(-1)
    if y.shape[0] != X.shape[0]:
      raise ValueError('labels must have num_rows entries')
    self.num_rows, self.num_features = X.shape
    self.prior_scale = float(prior_scale)
    ctx = _native.Context.current()
    h = ctypes.c_void_p()
    _native.check(_native.lib().gbm_target_logistic_regression(
        ctx.handle, _native.ptr(X),
        _native.DTYPE_BF16 if X.dtype == torch.bfloat16 else _native.DTYPE_F32,
        X.shape[0], X.shape[1], _native.ptr(y), self.prior_scale,
        _native.PRECISION_MIXED if precision == 'mixed' else _native.PRECISION_F32,
        ctypes.byref(h)), 'gbm_target_logistic_regression')
    self._handle = h
    self._ctx = ctx


class MultivariateNormalTriL(Target):
  """MultivariateNormalTriL(loc, scale_tril) (distributions/mvn_tril.py:44).

  L^-1 and the normalizer are formed once, in float64, at construction; the
  batched log-density -1/2 |L^-1 (x - loc)|^2 and gradient -L^-T L^-1 (x - loc)
  run on the device.
  """

  def __init__(self, loc, scale_tril):
    L = np.asarray(_util.as_tensor(scale_tril, torch.float64).cpu().numpy(), np.float64)
    mu = np.asarray(_util.as_tensor(loc, torch.float64).cpu().numpy(), np.float64).reshape(-1)
    d = L.shape[-1]
    if L.shape != (d, d) or mu.shape[0] != d:
      raise ValueError('scale_tril must be [D, D] and loc [D]')
    import scipy.linalg
    Linv = scipy.linalg.solve_triangular(np.tril(L), np.eye(d), lower=True)
    log_norm = -np.sum(np.log(np.abs(np.diag(L)))) - 0.5 * d * np.log(2 * np.pi)
    self.loc = mu
    ctx = _native.Context.current()
    loc_t = _util.as_tensor(mu, torch.float32)
    linv_t = _util.as_tensor(np.tril(Linv), torch.float32)
    h = ctypes.c_void_p()
    _native.check(_native.lib().gbm_target_mvn(ctx.handle, _native.ptr(loc_t), _native.ptr(linv_t),
                                               d, float(log_norm), ctypes.byref(h)),
                  'gbm_target_mvn')
    self._handle = h
    self._ctx = ctx
    # Device parameters, reused when the target joins a TargetBatch.
    self._loc_t, self._linv_t, self._log_norm, self.event_dim = loc_t, linv_t, float(log_norm), d


class NonCentredHierarchicalNormal(Target):
  """Non-centred hierarchical normal (eight-schools pattern,
  mcmc/eight_schools_hmc.py:41-58): state [mu, log tau, z_1..z_J]."""

  def __init__(self, y, sigma, mu_scale=5.0, tau_scale=5.0):
    y_t = _util.as_tensor(y, torch.float32).reshape(-1)
    s_t = _util.as_tensor(sigma, torch.float32).reshape(-1)
    if y_t.shape != s_t.shape:
      raise ValueError('y and sigma must have one entry per group')
    self.groups = y_t.shape[0]
    ctx = _native.Context.current()
    h = ctypes.c_void_p()
    _native.check(_native.lib().gbm_target_hierarchical_normal(
        ctx.handle, _native.ptr(y_t), _native.ptr(s_t), self.groups, float(mu_scale),
        float(tau_scale), ctypes.byref(h)), 'gbm_target_hierarchical_normal')
    self._handle = h
    self._ctx = ctx
    self._y_t, self._s_t = y_t, s_t
    self.mu_scale, self.tau_scale = float(mu_scale), float(tau_scale)
    self.event_dim = self.groups + 2


def resolve(target_log_prob_fn):
  """Return the engine target behind ``target_log_prob_fn`` or raise."""
  t = target_log_prob_fn
  if isinstance(t, Target):
    return t
  inner = getattr(t, '__self__', None)
  if isinstance(inner, Target):
    return inner
  raise NotImplementedError(
      'target_log_prob_fn must be one of the engine\'s built-in families '
      '(probability_gb300.targets.LogisticRegression, ...); arbitrary Python '
      'callables have no fused kernel and there is no autodiff fallback.')
