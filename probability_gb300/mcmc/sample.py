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
  if isinstance(first, (list, tuple)):
    if len(first) == 0:
      return first
    return type(first)(_stack([it[i] for it in items]) for i in range(len(first)))
  if isinstance(first, (int, float)):
    return torch.tensor(items)
  return items


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
