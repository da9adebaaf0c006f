"""HamiltonianMonteCarlo on the engine (reference: mcmc/hmc.py).

``HamiltonianMonteCarlo`` keeps the reference's structure and results:
MetropolisHastings(UncalibratedHamiltonianMonteCarlo) (hmc.py:439-448), so
``kernel_results.accepted_results.target_log_prob`` etc. work as before.  The
momentum draw, the L leapfrog steps with the fused target gradient, the
kinetic-energy correction and the MH test run as one device-side sequence
(``gbm_hmc_one_step``).  target_log_prob is float64 (the engine's energy
precision); states, gradients and momenta are float32.
"""
import ctypes

import torch

from probability_gb300 import _native, _util, targets
from probability_gb300.mcmc import kernel as kernel_base
from probability_gb300.mcmc.metropolis_hastings import MetropolisHastingsKernelResults

UncalibratedHamiltonianMonteCarloKernelResults = kernel_base.results_type(
    'UncalibratedHamiltonianMonteCarloKernelResults',
    ['log_acceptance_correction', 'target_log_prob', 'grads_target_log_prob',
     'initial_momentum', 'final_momentum', 'step_size', 'num_leapfrog_steps', 'seed'])


def _step_size_tensor(step_size, chains, dev):
  """Scalar -> float32 [1]; per-chain [C] or [C, 1] -> float32 [C]."""
  if isinstance(step_size, (list, tuple)):
    if len(step_size) != 1:
      raise ValueError('There should be exactly one `step_size` or it should '
                       'have same length as `current_state`.')
    step_size = step_size[0]
  s = _util.as_tensor(step_size, torch.float32, dev).reshape(-1)
  if s.numel() == 1:
    return s, 0
  if s.numel() != chains:
    raise ValueError('step_size must be a scalar or have one entry per chain')
  return s, 1


class _HmcEngine:
  """Owns the native HMC handle for one target, grown on demand."""

  def __init__(self, target):
    self.target = target
    self.handle = None
    self.capacity = 0

  def ensure(self, chains):
    if chains > self.capacity:
      if self.handle is not None:
        _native.lib().gbm_hmc_destroy(self.handle)
      h = ctypes.c_void_p()
      _native.check(_native.lib().gbm_hmc_create(self.target._handle, int(chains),
                                                 ctypes.byref(h)), 'gbm_hmc_create')
      self.handle, self.capacity = h, int(chains)

  def __del__(self):
    if self.handle is not None and _native._lib is not None:
      try:
        _native.lib().gbm_hmc_destroy(self.handle)
      except Exception:
        pass


def _hmc_transition(engine, state, target_log_prob, grads, step_size, num_leapfrog_steps, seed):
  q, layout, is_list = _util.flatten_state(state)
  C, D = q.shape
  dev = q.device
  engine.ensure(C)
  l0 = _util.as_tensor(target_log_prob, torch.float64, dev).reshape(C)
  g0, _, _ = _util.flatten_state(grads)
  eps, per_chain = _step_size_tensor(step_size, C, dev)
  f32 = lambda: torch.empty((C, D), dtype=torch.float32, device=dev)
  f64 = lambda: torch.empty(C, dtype=torch.float64, device=dev)
  out = dict(next_state=f32(), next_tlp=f64(), next_grads=f32(), proposed_state=f32(),
             proposed_tlp=f64(), proposed_grads=f32(), initial_momentum=f32(),
             final_momentum=f32(), corr=f64(), lar=f64(),
             is_accepted=torch.empty(C, dtype=torch.uint8, device=dev))
  P = _native.ptr
  _native.check(_native.lib().gbm_hmc_one_step(
      engine.handle, C, P(q), P(l0), P(g0), P(eps), per_chain, int(num_leapfrog_steps),
      _native.seed_words(seed), P(out['next_state']), P(out['next_tlp']),
      P(out['next_grads']), P(out['proposed_state']), P(out['proposed_tlp']),
      P(out['proposed_grads']), P(out['initial_momentum']), P(out['final_momentum']),
      P(out['corr']), P(out['lar']), P(out['is_accepted'])), 'gbm_hmc_one_step')
  unflat = lambda t: _util.unflatten_state(t, layout, is_list)
  out['is_accepted'] = out['is_accepted'].bool()
  return out, unflat, is_list


class UncalibratedHamiltonianMonteCarlo(kernel_base.TransitionKernel):
  """hmc.py:543-777: proposes by leapfrog integration, no MH correction."""

  def __init__(self, target_log_prob_fn, step_size, num_leapfrog_steps,
               state_gradients_are_stopped=False, store_parameters_in_results=False,
               experimental_shard_axis_names=None, name=None):
    self._target = targets.resolve(target_log_prob_fn)
    if experimental_shard_axis_names:
      raise NotImplementedError('the engine runs on one GPU; state sharding is not supported')
    self._parameters = dict(
        target_log_prob_fn=target_log_prob_fn, step_size=step_size,
        num_leapfrog_steps=num_leapfrog_steps,
        state_gradients_are_stopped=state_gradients_are_stopped, name=name,
        experimental_shard_axis_names=experimental_shard_axis_names,
        store_parameters_in_results=store_parameters_in_results)
    self._engine = _HmcEngine(self._target)

  target_log_prob_fn = property(lambda self: self._parameters['target_log_prob_fn'])
  step_size = property(lambda self: self._parameters['step_size'])
  num_leapfrog_steps = property(lambda self: self._parameters['num_leapfrog_steps'])
  state_gradients_are_stopped = property(
      lambda self: self._parameters['state_gradients_are_stopped'])
  name = property(lambda self: self._parameters['name'])

  @property
  def is_calibrated(self):
    return False

  def _params(self, pkr):
    if self._parameters['store_parameters_in_results']:
      return pkr.step_size, pkr.num_leapfrog_steps
    return self.step_size, self.num_leapfrog_steps

  def one_step(self, current_state, previous_kernel_results, seed=None):
    step_size, n = self._params(previous_kernel_results)
    seed = _util.sanitize_seed(seed)
    out, unflat, _ = _hmc_transition(
        self._engine, current_state, previous_kernel_results.target_log_prob,
        previous_kernel_results.grads_target_log_prob, step_size, int(n), seed)
    kr = previous_kernel_results._replace(
        log_acceptance_correction=out['corr'], target_log_prob=out['proposed_tlp'],
        grads_target_log_prob=unflat(out['proposed_grads']),
        initial_momentum=unflat(out['initial_momentum']),
        final_momentum=unflat(out['final_momentum']), seed=_util.seed_tensor(seed))
    return unflat(out['proposed_state']), kr

  def bootstrap_results(self, init_state):
    q, layout, is_list = _util.flatten_state(init_state)
    logp, grad = self._target.log_prob_and_grad(q)
    unflat = lambda t: _util.unflatten_state(t, layout, is_list)
    zeros = torch.zeros_like(q)
    r = UncalibratedHamiltonianMonteCarloKernelResults(
        log_acceptance_correction=torch.zeros_like(logp), target_log_prob=logp,
        grads_target_log_prob=unflat(grad), initial_momentum=unflat(zeros),
        final_momentum=unflat(zeros.clone()), step_size=[], num_leapfrog_steps=[],
        seed=_util.seed_tensor((0, 0)))
    if self._parameters['store_parameters_in_results']:
      r = r._replace(step_size=_util.as_tensor(self.step_size, torch.float32, q.device),
                     num_leapfrog_steps=int(self.num_leapfrog_steps))
    return r


class HamiltonianMonteCarlo(kernel_base.TransitionKernel):
  """hmc.py:175-540: MetropolisHastings(UncalibratedHamiltonianMonteCarlo)."""

  def __init__(self, target_log_prob_fn, step_size, num_leapfrog_steps,
               state_gradients_are_stopped=False, store_parameters_in_results=False,
               experimental_shard_axis_names=None, name=None):
    self._inner = UncalibratedHamiltonianMonteCarlo(
        target_log_prob_fn, step_size, num_leapfrog_steps, state_gradients_are_stopped,
        store_parameters_in_results, experimental_shard_axis_names, name or 'hmc_kernel')
    self._parameters = dict(self._inner.parameters)

  target_log_prob_fn = property(lambda self: self._inner.target_log_prob_fn)
  step_size = property(lambda self: self._inner.step_size)
  num_leapfrog_steps = property(lambda self: self._inner.num_leapfrog_steps)
  state_gradients_are_stopped = property(lambda self: self._inner.state_gradients_are_stopped)
  name = property(lambda self: self._inner.name)

  @property
  def is_calibrated(self):
    return True

  def one_step(self, current_state, previous_kernel_results, seed=None):
    """metropolis_hastings.py:160-254 around hmc.py:661-729, fused."""
    seed = _util.sanitize_seed(seed)
    prev = previous_kernel_results.accepted_results
    step_size, n = self._inner._params(prev)
    out, unflat, _ = _hmc_transition(
        self._inner._engine, current_state, prev.target_log_prob, prev.grads_target_log_prob,
        step_size, int(n), seed)
    proposed = prev._replace(
        log_acceptance_correction=out['corr'], target_log_prob=out['proposed_tlp'],
        grads_target_log_prob=unflat(out['proposed_grads']),
        initial_momentum=unflat(out['initial_momentum']),
        final_momentum=unflat(out['final_momentum']), seed=_util.seed_tensor(seed))
    acc = out['is_accepted']
    accepted = _choose(acc, proposed._replace(seed=[]), prev._replace(seed=[]))
    accepted = accepted._replace(target_log_prob=out['next_tlp'],
                                 grads_target_log_prob=unflat(out['next_grads']))
    kr = MetropolisHastingsKernelResults(
        accepted_results=accepted, is_accepted=acc, log_accept_ratio=out['lar'],
        proposed_state=unflat(out['proposed_state']), proposed_results=proposed, extra=[],
        seed=_util.seed_tensor(seed))
    return unflat(out['next_state']), kr

  def bootstrap_results(self, init_state):
    """metropolis_hastings.py:256-288."""
    pkr = self._inner.bootstrap_results(init_state)
    x = pkr.target_log_prob
    return MetropolisHastingsKernelResults(
        accepted_results=pkr._replace(seed=[]), is_accepted=torch.ones_like(x, dtype=torch.bool),
        log_accept_ratio=torch.zeros_like(x), proposed_state=init_state, proposed_results=pkr,
        extra=[], seed=_util.seed_tensor((0, 0)))


def _choose(is_accepted, proposed, current):
  """mcmc/internal/util.py:103-164: per-chain select over a results tuple."""
  def pick(p, c):
    if isinstance(p, torch.Tensor) and isinstance(c, torch.Tensor) and p.shape == c.shape \
        and p.dim() >= 1 and p.shape[0] == is_accepted.shape[0]:
      m = is_accepted.reshape((-1,) + (1,) * (p.dim() - 1))
      return torch.where(m, p, c)
    if isinstance(p, list) and isinstance(c, list) and len(p) == len(c) and p:
      return [pick(a, b) for a, b in zip(p, c)]
    return p
  return type(proposed)(*[pick(p, c) for p, c in zip(proposed, current)])
