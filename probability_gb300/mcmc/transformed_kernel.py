"""TransformedTransitionKernel on the engine (reference:
mcmc/transformed_kernel.py:165-500).

The inner kernel (HamiltonianMonteCarlo, NoUTurnSampler, optionally inside
DualAveragingStepSizeAdaptation) samples an unconstrained state x; its
target is the engine's target seen through the bijectors (C ABI
gbm_target_transformed): log p(f(x)) + log |f'(x)| with the chain rule in
the gradient, fused around the wrapped target's kernels.  Same constructor,
``one_step`` / ``bootstrap_results`` contract and results type as the
reference: ``TransformedTransitionKernelResults(transformed_state,
inner_results)``, and ``one_step`` continues from
``previous_kernel_results.transformed_state``.
"""
import ctypes

import numpy as np
import torch

from probability_gb300 import _native, _util, bijectors as tfb, targets
from probability_gb300.mcmc import kernel as kernel_base

TransformedTransitionKernelResults = kernel_base.results_type(
    'TransformedTransitionKernelResults', ['transformed_state', 'inner_results'])


class TransformedTarget(targets.Target):
  """``inner`` (an engine target) seen through one bijector per dimension."""

  def __init__(self, inner, codes):
    self.inner = inner
    codes = np.ascontiguousarray(codes, dtype=np.int32)
    h = ctypes.c_void_p()
    _native.check(_native.lib().gbm_target_transformed(
        inner._handle, codes.ctypes.data_as(ctypes.c_void_p), ctypes.byref(h)),
        'gbm_target_transformed')
    self._handle = h
    self._ctx = inner._ctx
    self.codes = codes


def _find_target(kernel):
  """transformed_kernel.py:105-123: the nested target_log_prob_fn."""
  p = kernel.parameters
  if 'target_log_prob_fn' in p:
    return targets.resolve(p['target_log_prob_fn'])
  if 'inner_kernel' in p:
    return _find_target(p['inner_kernel'])
  raise ValueError('inner_kernel has no target_log_prob_fn')


def _update_target(kernel, target):
  """transformed_kernel.py:126-145: a copy of the kernel stack with a new target."""
  p = kernel.parameters
  if 'target_log_prob_fn' in p:
    return kernel.copy(target_log_prob_fn=target)
  return kernel.copy(inner_kernel=_update_target(p['inner_kernel'], target))


class TransformedTransitionKernel(kernel_base.TransitionKernel):
  """transformed_kernel.py:165: samples `inner_kernel` in the unconstrained
  space of `bijector` (one elementwise bijector, or one per state part)."""

  def __init__(self, inner_kernel, bijector, name=None):
    self._parameters = dict(inner_kernel=inner_kernel, bijector=bijector,
                            name=name or 'transformed_kernel')
    self._base_target = _find_target(inner_kernel)
    self._kernel = None          # built on first use, once the part sizes are known
    self._part_dims = None

  inner_kernel = property(lambda self: self._parameters['inner_kernel'])
  bijector = property(lambda self: self._parameters['bijector'])
  name = property(lambda self: self._parameters['name'])

  @property
  def is_calibrated(self):
    return self.inner_kernel.is_calibrated

  def _bijectors(self, nparts):
    b = self.bijector
    bl = list(b) if isinstance(b, (list, tuple)) else [b] * nparts
    if len(bl) != nparts:
      raise ValueError('need one bijector per state part (%d), got %d' % (nparts, len(bl)))
    for x in bl:
      if not isinstance(x, tfb.Bijector):
        raise NotImplementedError('bijectors are probability_gb300.bijectors Identity, Exp, '
                                  'Softplus or Sigmoid')
    return bl

  def _ensure(self, state):
    parts = state if isinstance(state, (list, tuple)) else [state]
    dims = [int(np.prod(p.shape[1:])) if p.dim() > 1 else 1 for p in
            (_util.as_tensor(x, torch.float32) for x in parts)]
    if self._kernel is not None:
      if dims != self._part_dims:
        raise ValueError('state parts changed shape')
      return
    bl = self._bijectors(len(parts))
    codes = np.concatenate([np.full(d, b.code, np.int32) for d, b in zip(dims, bl)])
    if codes.shape[0] != self._base_target.dim:
      raise ValueError('state has %d dimensions, the target %d' % (codes.shape[0],
                                                                  self._base_target.dim))
    self._part_dims = dims
    self._target = TransformedTarget(self._base_target, codes)
    self._kernel = _update_target(self.inner_kernel, self._target)

  def _map(self, state, fn_name):
    parts = state if isinstance(state, (list, tuple)) else [state]
    bl = self._bijectors(len(parts))
    out = [getattr(b, fn_name)(_util.as_tensor(x, torch.float32)) for b, x in zip(bl, parts)]
    return out if isinstance(state, (list, tuple)) else out[0]

  def one_step(self, current_state, previous_kernel_results, seed=None):
    xt = previous_kernel_results.transformed_state
    self._ensure(xt)
    xt_next, kr = self._kernel.one_step(xt, previous_kernel_results.inner_results, seed=seed)
    return (self._map(xt_next, 'forward'),
            TransformedTransitionKernelResults(transformed_state=xt_next, inner_results=kr))

  def bootstrap_results(self, init_state=None, transformed_init_state=None):
    if (init_state is None) == (transformed_init_state is None):
      raise ValueError('Must specify exactly one of `init_state` or `transformed_init_state`.')
    xt = (self._map(init_state, 'inverse') if transformed_init_state is None
          else transformed_init_state)
    self._ensure(xt)
    return TransformedTransitionKernelResults(
        transformed_state=xt, inner_results=self._kernel.bootstrap_results(xt))
