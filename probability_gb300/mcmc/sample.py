"""sample_chain (reference: mcmc/sample.py:81-383).

Same signature, step schedule and return types.  Transition t uses the key
``gbm_step_key(seed, t)`` (a Philox stream addressed by step, replacing the
reference's split-per-step seed chain); the key is recorded in each kernel
result's ``seed`` field, so ``kernel.one_step(state, results, seed=...)``
replays a transition exactly.  All chain state stays on the device; the
host loop only launches transitions.
"""
import collections
import warnings

import numpy as np
import torch

from probability_gb300 import _util

StatesAndTrace = collections.namedtuple('StatesAndTrace', ['all_states', 'trace'])
CheckpointableStatesAndTrace = collections.namedtuple(
    'CheckpointableStatesAndTrace', ['all_states', 'trace', 'final_kernel_results'])


def _trace_kernel_results(states, kernel_results):
  return kernel_results


def _stack(items):
  first = items[0]
  if isinstance(first, torch.Tensor):
    return torch.stack(items)
  if isinstance(first, tuple) and hasattr(first, '_fields'):
    return type(first)(*[_stack([it[i] for it in items]) for i in range(len(first))])
  if isinstance(first, dict):
    return {k: _stack([it[k] for it in items]) for k in first}
  if isinstance(first, (list, tuple)):
    if len(first) == 0:
      return first
    return type(first)(_stack([it[i] for it in items]) for i in range(len(first)))
  if isinstance(first, (int, float)):
    return torch.tensor(items)
  return items


ChainRun = collections.namedtuple(
    'ChainRun', ['all_states', 'trace', 'final_state', 'final_step_size', 'final_da_state'])


def _unwrap(kernel):
  """(sampler, dual-averaging kernel or None) for the engine's kernels."""
  from probability_gb300.mcmc.dual_averaging_step_size_adaptation import (
      DualAveragingStepSizeAdaptation)
  from probability_gb300.mcmc.hmc import HamiltonianMonteCarlo
  from probability_gb300.mcmc.nuts import NoUTurnSampler
  from probability_gb300.mcmc.dual_averaging_step_size_adaptation import reduce_logmeanexp
  da = None
  if isinstance(kernel, DualAveragingStepSizeAdaptation):
    if kernel.parameters['reduce_fn'] is not reduce_logmeanexp:
      # The device loop's adaptation reduces with reduce_logmeanexp.
      return None, None
    da, kernel = kernel, kernel.inner_kernel
  if isinstance(kernel, (NoUTurnSampler, HamiltonianMonteCarlo)):
    return kernel, da
  return None, None


def run_chain(kernel, num_results, current_state, num_burnin_steps=0,
              num_steps_between_results=0, seed=None, first_step=0, step_size=None,
              da_state=None, free_running_draws=False):
  """Device-resident ``sample_chain`` for the engine's NUTS / HMC kernels
  (optionally inside DualAveragingStepSizeAdaptation): the whole loop, the
  adaptation and the trace run in C++ on the device (gbm_*_sample_chain).

  free_running_draws (NUTS): the results drawn at the final step size (past
  the adaptation window, no thinning) come from the free-running loop
  (gbm_nuts_set_free_running): per chain the same transitions, without
  waiting for the batch's longest trajectory.

  Returns ChainRun(all_states [R, C, D], trace dict, final_state,
  final_step_size, final_da_state); pass the last three back (with
  first_step advanced) to continue the same chain.
  """
  import torch
  from probability_gb300 import _native
  from probability_gb300.mcmc.hmc import HamiltonianMonteCarlo, _step_size_tensor
  sampler, da = _unwrap(kernel)
  if sampler is None:
    raise NotImplementedError('run_chain needs the engine\'s NoUTurnSampler or '
                              'HamiltonianMonteCarlo, optionally in DualAveragingStepSizeAdaptation')
  seed = _util.sanitize_seed(seed)
  q, layout, is_list = _util.flatten_state(current_state)
  q = q.clone()
  C, D = q.shape
  dev = q.device
  is_hmc = isinstance(sampler, HamiltonianMonteCarlo)
  target = sampler._inner._target if is_hmc else sampler._target
  logp, grad = target.log_prob_and_grad(q)
  eps0 = sampler.step_size if step_size is None else step_size
  eps, per_chain = _step_size_tensor(eps0, C, dev)
  eps = eps.clone()
  groups = eps.numel()
  if da is not None and da_state is None:
    da_state = torch.zeros((groups, 4), dtype=torch.float64, device=dev)
    st = da.parameters['shrinkage_target']
    base = eps.to(torch.float64) if st is None else _util.as_tensor(st, torch.float64, dev)
    da_state[:, 2] = (float(np.log(10.)) if st is None else 0.0) + torch.log(base).reshape(-1)
  R = int(num_results)
  f32 = lambda *s: torch.empty(s, dtype=torch.float32, device=dev)
  tr = dict(state=f32(R, C, D), target_log_prob=torch.empty((R, C), dtype=torch.float64, device=dev),
            log_accept_ratio=torch.empty((R, C), dtype=torch.float64, device=dev),
            is_accepted=torch.empty((R, C), dtype=torch.uint8, device=dev),
            step_size=f32(R, groups))
  if not is_hmc:
    tr['leapfrogs_taken'] = torch.empty((R, C), dtype=torch.int32, device=dev)
    tr['has_divergence'] = torch.empty((R, C), dtype=torch.uint8, device=dev)
  P = _native.ptr
  n_adapt = int(da.num_adaptation_steps) if da is not None else 0
  dap = da.parameters if da is not None else {}
  tap = float(np.asarray(dap.get('target_accept_prob', 0.75)).reshape(-1)[0])
  args = (n_adapt, tap, float(dap.get('exploration_shrinkage', 0.05)),
          float(dap.get('step_count_smoothing', 10)), float(dap.get('decay_rate', 0.75)),
          P(da_state) if da is not None else None)
  if is_hmc:
    eng = sampler._inner._engine
    eng.ensure(C)
    _native.check(_native.lib().gbm_hmc_sample_chain(
        eng.handle, C, P(q), P(logp), P(grad), P(eps), per_chain,
        int(sampler.num_leapfrog_steps), _native.seed_words(seed), int(first_step), R,
        int(num_burnin_steps), int(num_steps_between_results), *args, P(tr['state']),
        P(tr['target_log_prob']), P(tr['log_accept_ratio']), P(tr['is_accepted']),
        P(tr['step_size'])), 'gbm_hmc_sample_chain')
  else:
    sampler._ensure(C)
    lib = _native.lib()
    _native.check(lib.gbm_nuts_set_free_running(sampler._handle, int(bool(free_running_draws))),
                  'gbm_nuts_set_free_running')
    try:
      _native.check(lib.gbm_nuts_sample_chain(
          sampler._handle, C, P(q), P(logp), P(grad), P(eps), per_chain,
          _native.seed_words(seed), int(first_step), R, int(num_burnin_steps),
          int(num_steps_between_results), *args, P(tr['state']), P(tr['target_log_prob']),
          P(tr['log_accept_ratio']), P(tr['leapfrogs_taken']), P(tr['is_accepted']),
          P(tr['has_divergence']), P(tr['step_size'])), 'gbm_nuts_sample_chain')
    finally:
      lib.gbm_nuts_set_free_running(sampler._handle, 0)
  for k in ('is_accepted', 'has_divergence'):
    if k in tr:
      tr[k] = tr[k].bool()
  states = tr.pop('state')
  all_states = (_util.unflatten_state(states.reshape(R * C, D), layout, is_list)
                if is_list else states.reshape((R,) + tuple(layout[1][0])))
  return ChainRun(all_states, tr, _util.unflatten_state(q, layout, is_list), eps, da_state)


def sample_chain(num_results, current_state, previous_kernel_results=None, kernel=None,
                 num_burnin_steps=0, num_steps_between_results=0,
                 trace_fn=_trace_kernel_results, return_final_kernel_results=False,
                 parallel_iterations=10, seed=None, name=None):
  """Runs ``1 + num_burnin_steps`` transitions before result 0 and
  ``1 + num_steps_between_results`` before each later result
  (sample.py:359-367)."""
  if kernel is None:
    raise ValueError('kernel must be provided')
  is_seeded = seed is not None
  seed = _util.sanitize_seed(seed)
  if not kernel.is_calibrated:
    warnings.warn('supplied `TransitionKernel` is not calibrated. Markov '
                  'chain may not converge to intended target distribution.')
  num_results = int(num_results)
  num_burnin_steps = int(num_burnin_steps)
  num_steps_between_results = int(num_steps_between_results)
  if (trace_fn is None and previous_kernel_results is None and not return_final_kernel_results
      and is_seeded and _unwrap(kernel)[0] is not None
      and not isinstance(current_state, (list, tuple))):
    # Nothing to trace in Python: run the whole loop on the device.
    return run_chain(kernel, num_results, current_state, num_burnin_steps,
                     num_steps_between_results, seed=seed).all_states
  if previous_kernel_results is None:
    previous_kernel_results = kernel.bootstrap_results(current_state)
  no_trace = trace_fn is None
  if no_trace:
    trace_fn = lambda *args: ()
  state, kr = current_state, previous_kernel_results
  states, traces = [], []
  t = 0
  for i in range(num_results):
    n = (1 + num_burnin_steps) if i == 0 else (1 + num_steps_between_results)
    for _ in range(n):
      key = _util.step_key(seed, t) if is_seeded else None
      state, kr = kernel.one_step(state, kr, seed=key)
      t += 1
    states.append(state)
    traces.append(trace_fn(state, kr))
  all_states = _stack(states) if states else []
  trace = _stack(traces) if traces else []
  if return_final_kernel_results:
    return CheckpointableStatesAndTrace(all_states=all_states, trace=trace,
                                        final_kernel_results=kr)
  return all_states if no_trace else StatesAndTrace(all_states=all_states, trace=trace)
