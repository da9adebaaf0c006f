"""DualAveragingStepSizeAdaptation on the engine
(reference: mcmc/dual_averaging_step_size_adaptation.py).

Same constructor and ``DualAveragingStepSizeAdaptationResults`` fields.  The
update (reduce_logmeanexp over chains, error sum, shrinkage, averaging,
freeze after ``num_adaptation_steps``) runs in one device kernel
(``gbm_dual_averaging_update``); the step size never leaves the device.
"""
import numpy as np
import torch

from probability_gb300 import _native, _util
from probability_gb300.mcmc import kernel as kernel_base
from probability_gb300.mcmc import simple_step_size_adaptation as ssa

DualAveragingStepSizeAdaptationResults = kernel_base.results_type(
    'DualAveragingStepSizeAdaptationResults',
    ['inner_results', 'target_accept_prob', 'log_shrinkage_target', 'exploration_shrinkage',
     'step_count_smoothing', 'decay_rate', 'error_sum', 'log_averaging_step', 'step',
     'num_adaptation_steps', 'new_step_size'])


def reduce_logmeanexp(input_tensor, axis=None, keepdims=False, experimental_named_axis=None):
  """log(mean(exp(x))) over `axis` (math/generic.py:221-275).  The default
  reduction; for the engine's kernels the dual-averaging kernel performs it
  on the device itself."""
  if experimental_named_axis:
    raise NotImplementedError('the engine runs on one GPU; no named-axis reduction')
  x = torch.as_tensor(input_tensor)
  dims = tuple(range(x.dim())) if axis is None else tuple(np.atleast_1d(axis).tolist())
  if not dims:
    return x
  n = int(np.prod([x.shape[a] for a in dims]))
  m = torch.amax(x, dim=dims, keepdim=True)
  m = torch.where(torch.isfinite(m), m, torch.zeros_like(m))
  out = torch.log(torch.sum(torch.exp(x - m), dim=dims, keepdim=True)) + m - np.log(n)
  return out if keepdims else out.reshape([s for i, s in enumerate(x.shape) if i not in dims])


def reduce_log_harmonic_mean_exp(input_tensor, axis=None, keepdims=False,
                                 experimental_named_axis=None):
  """log(1 / mean(1 / exp(x))) = -reduce_logmeanexp(-x) (math/generic.py:
  387-428): the reduction the reference recommends for dual averaging when
  some chains may be stuck (dual_averaging_step_size_adaptation.py:135-143)."""
  return -reduce_logmeanexp(-torch.as_tensor(input_tensor), axis=axis, keepdims=keepdims,
                            experimental_named_axis=experimental_named_axis)


def _enable_store_parameters_in_results(kernel):
  """mcmc/internal/util.py:311-345."""
  p = getattr(kernel, 'parameters', {})
  if 'store_parameters_in_results' in p and not p['store_parameters_in_results']:
    return kernel.copy(store_parameters_in_results=True)
  if 'inner_kernel' in p:
    inner = _enable_store_parameters_in_results(p['inner_kernel'])
    if inner is not p['inner_kernel']:
      return kernel.copy(inner_kernel=inner)
  return kernel


class DualAveragingStepSizeAdaptation(kernel_base.TransitionKernel):
  """dual_averaging_step_size_adaptation.py:74-627."""

  def __init__(self, inner_kernel, num_adaptation_steps, target_accept_prob=0.75,
               exploration_shrinkage=0.05, shrinkage_target=None, step_count_smoothing=10,
               decay_rate=0.75, step_size_setter_fn=ssa.hmc_like_step_size_setter_fn,
               step_size_getter_fn=ssa.hmc_like_step_size_getter_fn,
               log_accept_prob_getter_fn=ssa.hmc_like_log_accept_prob_getter_fn,
               reduce_fn=reduce_logmeanexp, experimental_reduce_chain_axis_names=None,
               validate_args=False, name=None):
    inner_kernel = _enable_store_parameters_in_results(inner_kernel)
    if validate_args:
      tap = np.asarray(target_accept_prob, np.float64)
      if np.any(tap <= 0):
        raise ValueError('`target_accept_prob` must be > 0.')
      if np.any(tap >= 1):
        raise ValueError('`target_accept_prob` must be < 1.')
    if experimental_reduce_chain_axis_names:
      raise NotImplementedError('the engine runs on one GPU; no cross-device chain reduction')
    self._parameters = dict(
        inner_kernel=inner_kernel, num_adaptation_steps=num_adaptation_steps,
        target_accept_prob=target_accept_prob, exploration_shrinkage=exploration_shrinkage,
        shrinkage_target=shrinkage_target, step_count_smoothing=step_count_smoothing,
        decay_rate=decay_rate, step_size_setter_fn=step_size_setter_fn,
        step_size_getter_fn=step_size_getter_fn,
        log_accept_prob_getter_fn=log_accept_prob_getter_fn, reduce_fn=reduce_fn,
        experimental_reduce_chain_axis_names=experimental_reduce_chain_axis_names,
        validate_args=validate_args, name=name)

  inner_kernel = property(lambda self: self._parameters['inner_kernel'])
  num_adaptation_steps = property(lambda self: self._parameters['num_adaptation_steps'])
  name = property(lambda self: self._parameters['name'])

  def step_size_setter_fn(self, kernel_results, new_step_size):
    return self._parameters['step_size_setter_fn'](kernel_results, new_step_size)

  def step_size_getter_fn(self, kernel_results):
    return self._parameters['step_size_getter_fn'](kernel_results)

  def log_accept_prob_getter_fn(self, kernel_results):
    return self._parameters['log_accept_prob_getter_fn'](kernel_results)

  @property
  def is_calibrated(self):
    return self.inner_kernel.is_calibrated

  def one_step(self, current_state, previous_kernel_results, seed=None):
    pkr = previous_kernel_results
    inner_results = self.step_size_setter_fn(pkr.inner_results, pkr.new_step_size)  # :482-485
    kwargs = {} if seed is None else dict(seed=seed)
    new_state, new_inner = self.inner_kernel.one_step(current_state, inner_results, **kwargs)
    lap = self.log_accept_prob_getter_fn(new_inner).to(torch.float64).contiguous()
    step_size = self.step_size_getter_fn(new_inner)
    eps = _util.as_tensor(step_size, torch.float32, lap.device).reshape(-1).clone()
    groups = eps.numel()
    per_chain = 1 if groups > 1 else 0
    if per_chain and groups != lap.numel():
      raise ValueError('per-chain step sizes need one log_accept_prob per chain')
    state = torch.stack([
        _util.as_tensor(pkr.error_sum, torch.float64, lap.device).reshape(-1).expand(groups),
        _util.as_tensor(pkr.log_averaging_step, torch.float64, lap.device).reshape(-1).expand(groups),
        _util.as_tensor(pkr.log_shrinkage_target, torch.float64, lap.device).reshape(-1).expand(groups),
        torch.full((groups,), float(pkr.step), dtype=torch.float64, device=lap.device)], 1)
    state = state.contiguous()
    tap = pkr.target_accept_prob
    tap_t = None
    if isinstance(tap, torch.Tensor) and tap.numel() > 1:
      tap_t = tap.to(lap.device, torch.float64).reshape(-1).contiguous()
      tap_scalar = 0.0
    else:
      tap_scalar = float(tap)
    ctx = _native.Context.current()
    P = _native.ptr
    reduce_fn = self._parameters['reduce_fn']
    if reduce_fn is reduce_logmeanexp or per_chain:
      # The chain reduction (reduce_logmeanexp over the chain axis, or none
      # for per-chain step sizes, :410-422) runs inside the kernel.
      _native.check(_native.lib().gbm_dual_averaging_update(
          ctx.handle, lap.numel(), P(lap), per_chain, int(pkr.num_adaptation_steps),
          tap_scalar, P(tap_t), float(pkr.exploration_shrinkage),
          float(pkr.step_count_smoothing), float(pkr.decay_rate), P(state), P(eps)),
          'gbm_dual_averaging_update')
    else:
      # A custom reduce_fn (:141, 410-422) over the chain axis of the log
      # accept probabilities min(lar, 0), non-finite -> -inf
      # (simple_step_size_adaptation.py:42-48), on the device.
      lp = torch.where(torch.isfinite(lap), lap, torch.full_like(lap, -np.inf)).clamp(max=0.0)
      try:
        red = reduce_fn(lp, axis=0, keepdims=False, experimental_named_axis=None)
      except TypeError:
        red = reduce_fn(lp, axis=0, keepdims=False)
      red = _util.as_tensor(red, torch.float64, lap.device).reshape(-1).contiguous()
      _native.check(_native.lib().gbm_dual_averaging_update_reduced(
          ctx.handle, 1, P(red), int(pkr.num_adaptation_steps), tap_scalar, P(tap_t),
          float(pkr.exploration_shrinkage), float(pkr.step_count_smoothing),
          float(pkr.decay_rate), P(state), P(eps)), 'gbm_dual_averaging_update_reduced')
    shape = tuple(torch.as_tensor(step_size).shape) if not isinstance(step_size, torch.Tensor) \
        else tuple(step_size.shape)
    new_step = eps.reshape(shape)
    sq = (lambda t: t.reshape(shape))
    return new_state, pkr._replace(
        inner_results=new_inner, error_sum=sq(state[:, 0]), step=pkr.step + 1,
        log_averaging_step=sq(state[:, 1]), new_step_size=new_step)

  def bootstrap_results(self, init_state):
    return self._bootstrap_from_inner_results(init_state,
                                              self.inner_kernel.bootstrap_results(init_state))

  def _bootstrap_from_inner_results(self, init_state, inner_results):
    """:546-609: fresh adaptation state around existing inner results."""
    step_size = self.step_size_getter_fn(inner_results)
    dev = _util.device()
    s = _util.as_tensor(step_size, torch.float32, dev)
    st = self._parameters['shrinkage_target']
    if st is None:
      log_shrink = float(np.log(10.)) + torch.log(s.to(torch.float64))     # :588-590
    else:
      log_shrink = torch.log(_util.as_tensor(st, torch.float64, dev)).expand(s.shape).clone()
    tap = self._parameters['target_accept_prob']
    tap = tap if isinstance(tap, (float, int)) else _util.as_tensor(tap, torch.float64, dev)
    return DualAveragingStepSizeAdaptationResults(
        inner_results=inner_results, target_accept_prob=tap,
        log_shrinkage_target=log_shrink,
        exploration_shrinkage=float(self._parameters['exploration_shrinkage']),
        step_count_smoothing=float(self._parameters['step_count_smoothing']),
        decay_rate=float(self._parameters['decay_rate']),
        error_sum=torch.zeros_like(s, dtype=torch.float64),
        log_averaging_step=torch.zeros_like(s, dtype=torch.float64), step=0,
        num_adaptation_steps=int(self.num_adaptation_steps), new_step_size=s)
