"""NoUTurnSampler on the engine (reference: mcmc/nuts.py).

Same constructor, ``one_step``/``bootstrap_results`` contract and
``NUTSKernelResults`` fields as the reference (nuts.py:74-91, 197-503).  The
whole transition -- momentum draw, iterative tree doubling with the
precomputed U-turn slot tables, fused leapfrog + target gradient per leaf,
multinomial sampling with float64 log-weights -- runs in the engine
(``gbm_nuts_one_step``).  target_log_prob and energy are float64.
"""
import collections
import ctypes

import numpy as np
import torch

from probability_gb300 import _native, _util, targets
from probability_gb300.mcmc import kernel as kernel_base
from probability_gb300.mcmc.hmc import _step_size_tensor

NUTSKernelResults = kernel_base.results_type('NUTSKernelResults', [
    'target_log_prob', 'grads_target_log_prob', 'step_size', 'log_accept_ratio',
    'leapfrogs_taken', 'is_accepted', 'reach_max_depth', 'has_divergence', 'energy', 'seed'])


def build_tree_uturn_instruction(max_depth, init_memory=0):
  """nuts.py:1013-1028 (host, at construction): the (first, last) leaf of
  every internal node of a depth-``max_depth`` tree, leaves numbered from
  ``init_memory + 1``."""
  pairs = set()
  for h in range(1, max_depth + 1):
    size = 1 << h
    for a in range(0, 1 << max_depth, size):
      pairs.add((a + init_memory + 1, a + init_memory + size))
  return np.array(sorted(pairs), dtype=np.int32).reshape(-1, 2)


def generate_efficient_write_read_instruction(instruction_array):
  """nuts.py:1031-1071: per-leaf write slot and U-turn read range.  A leaf
  that starts a subtree keeps (momentum, cumsum) alive until the subtree's
  last leaf; its slot is the number of such live leaves minus one; leaves
  that start nothing write a dummy slot (the maximum live count)."""
  n = int(np.max(instruction_array)) + 1
  last_end = np.full(n, -1)
  ends_at = [[] for _ in range(n)]
  for a, b in instruction_array:
    last_end[a] = max(last_end[a], b)
    ends_at[b].append(a)
  alive = [[i for i in range(j + 1) if last_end[i] >= j] for j in range(n)]
  live = np.array([len(a) for a in alive])
  write = live - 1
  write[last_end < 0] = live.max()
  read = []
  for j in range(n):
    if ends_at[j]:
      r0 = alive[j].index(min(ends_at[j]))
      read.append([r0, r0 + len(ends_at[j])])
    else:
      read.append([0, 0])
  return write, np.asarray(read)


FreeRun = collections.namedtuple(
    'FreeRun', ['all_states', 'trace', 'transitions_done', 'leaf_iterations'])


def run_free(handle, q, kr, step_size, per_chain, seed, first_step, transitions_per_chain,
             max_leaf_iterations, state_shape):
  """gbm_nuts_run_free for a sampler handle: q [elements] float32 on the
  device, kr the results carrying target_log_prob / grads_target_log_prob.
  Returns FreeRun(all_states [K, *state_shape], trace of [K, C] tensors,
  transitions_done [C], leaf_iterations)."""
  dev = q.device
  C = kr.target_log_prob.numel()
  K = int(transitions_per_chain)
  E = q.numel()
  tr = dict(target_log_prob=torch.empty((K, C), dtype=torch.float64, device=dev),
            log_accept_ratio=torch.empty((K, C), dtype=torch.float64, device=dev),
            leapfrogs_taken=torch.zeros((K, C), dtype=torch.int32, device=dev),
            is_accepted=torch.zeros((K, C), dtype=torch.uint8, device=dev),
            has_divergence=torch.zeros((K, C), dtype=torch.uint8, device=dev))
  states = torch.empty((K, E), dtype=torch.float32, device=dev)
  done = torch.empty(C, dtype=torch.int32, device=dev)
  l0 = _util.as_tensor(kr.target_log_prob, torch.float64, dev).reshape(C).contiguous()
  g0 = _util.as_tensor(kr.grads_target_log_prob, torch.float32, dev).reshape(-1).contiguous()
  iters = ctypes.c_int64()
  P = _native.ptr
  _native.check(_native.lib().gbm_nuts_run_free(
      handle, C, P(q), P(l0), P(g0), P(step_size), per_chain, _native.seed_words(seed),
      int(first_step), K, int(max_leaf_iterations), P(done), P(states),
      P(tr['target_log_prob']), P(tr['log_accept_ratio']), P(tr['leapfrogs_taken']),
      P(tr['is_accepted']), P(tr['has_divergence']), ctypes.byref(iters)), 'gbm_nuts_run_free')
  for k in ('is_accepted', 'has_divergence'):
    tr[k] = tr[k].bool()
  return FreeRun(states.reshape((K,) + tuple(state_shape)), tr, done, int(iters.value))


class NoUTurnSampler(kernel_base.TransitionKernel):
  """nuts.py:165-946 (multinomial sampling, generalised U-turn)."""

  def __init__(self, target_log_prob_fn, step_size, max_tree_depth=10,
               max_energy_diff=1000., unrolled_leapfrog_steps=1, parallel_iterations=10,
               experimental_shard_axis_names=None, name=None):
    if max_tree_depth is None or int(max_tree_depth) < 1:
      raise ValueError('max_tree_depth must be known statically and >= 1 but was '
                       '{}'.format(max_tree_depth))
    if experimental_shard_axis_names:
      raise NotImplementedError('the engine runs on one GPU; state sharding is not supported')
    self._target = targets.resolve(target_log_prob_fn)
    self._max_tree_depth = int(max_tree_depth)
    instr = build_tree_uturn_instruction(self._max_tree_depth, init_memory=-1)
    self._write_instruction, self._read_instruction = \
        generate_efficient_write_read_instruction(instr)
    self._parameters = dict(
        target_log_prob_fn=target_log_prob_fn, step_size=step_size,
        max_tree_depth=self._max_tree_depth, max_energy_diff=max_energy_diff,
        unrolled_leapfrog_steps=unrolled_leapfrog_steps,
        parallel_iterations=parallel_iterations,
        experimental_shard_axis_names=experimental_shard_axis_names, name=name)
    self._handle = None
    self._capacity = 0
    self.last_leaf_iterations = 0

  target_log_prob_fn = property(lambda self: self._parameters['target_log_prob_fn'])
  step_size = property(lambda self: self._parameters['step_size'])
  max_tree_depth = property(lambda self: self._max_tree_depth)
  max_energy_diff = property(lambda self: self._parameters['max_energy_diff'])
  unrolled_leapfrog_steps = property(lambda self: self._parameters['unrolled_leapfrog_steps'])
  parallel_iterations = property(lambda self: self._parameters['parallel_iterations'])
  name = property(lambda self: self._parameters['name'])
  write_instruction = property(lambda self: self._write_instruction)
  read_instruction = property(lambda self: self._read_instruction)

  @property
  def is_calibrated(self):
    return True

  def _ensure(self, chains):
    if chains > self._capacity:
      if self._handle is not None:
        _native.lib().gbm_nuts_destroy(self._handle)
      h = ctypes.c_void_p()
      _native.check(_native.lib().gbm_nuts_create(
          self._target._handle, int(chains), self._max_tree_depth,
          float(self.max_energy_diff), int(self.unrolled_leapfrog_steps), ctypes.byref(h)),
          'gbm_nuts_create')
      self._handle, self._capacity = h, int(chains)

  def __del__(self):
    if getattr(self, '_handle', None) is not None and _native._lib is not None:
      try:
        _native.lib().gbm_nuts_destroy(self._handle)
      except Exception:
        pass

  def one_step(self, current_state, previous_kernel_results, seed=None):
    seed = _util.sanitize_seed(seed)
    q, layout, is_list = _util.flatten_state(current_state)
    C, D = q.shape
    dev = q.device
    self._ensure(C)
    pkr = previous_kernel_results
    l0 = _util.as_tensor(pkr.target_log_prob, torch.float64, dev).reshape(C)
    g0, _, _ = _util.flatten_state(pkr.grads_target_log_prob)
    eps, per_chain = _step_size_tensor(pkr.step_size, C, dev)
    nq = torch.empty_like(q)
    ng = torch.empty_like(q)
    f64 = lambda: torch.empty(C, dtype=torch.float64, device=dev)
    u8 = lambda: torch.empty(C, dtype=torch.uint8, device=dev)
    nl, lar, energy = f64(), f64(), f64()
    lf = torch.empty(C, dtype=torch.int32, device=dev)
    acc, rmd, div = u8(), u8(), u8()
    P = _native.ptr
    _native.check(_native.lib().gbm_nuts_one_step(
        self._handle, C, P(q), P(l0), P(g0), P(eps), per_chain, _native.seed_words(seed),
        P(nq), P(nl), P(ng), P(lar), P(lf), P(acc), P(rmd), P(div), P(energy), None),
        'gbm_nuts_one_step')
    n = ctypes.c_int64()
    _native.lib().gbm_nuts_last_leaf_iterations(self._handle, ctypes.byref(n))
    self.last_leaf_iterations = int(n.value)
    unflat = lambda t: _util.unflatten_state(t, layout, is_list)
    kr = NUTSKernelResults(
        target_log_prob=nl, grads_target_log_prob=unflat(ng), step_size=pkr.step_size,
        log_accept_ratio=lar, leapfrogs_taken=lf, is_accepted=acc.bool(),
        reach_max_depth=rmd.bool(), has_divergence=div.bool(), energy=energy,
        seed=_util.seed_tensor(seed))
    return unflat(nq), kr

  def run_free(self, current_state, kernel_results, transitions_per_chain, seed,
               first_step=0, max_leaf_iterations=1 << 40):
    """Free-running transitions: every chain runs `transitions_per_chain`
    one_step transitions with keys step_key(seed, first_step + t) (the
    transitions sample_chain runs at a fixed step size), each chain starting
    its next transition as soon as its own trajectory ends (no lock-step);
    per chain equal to one_step with the same keys.  At most
    `max_leaf_iterations` leapfrog steps per chain.  Returns
    FreeRun(all_states [K, C, D], trace, transitions_done, leaf_iterations)."""
    q, layout, is_list = _util.flatten_state(current_state)
    if is_list:
      raise NotImplementedError('run_free takes a single-part state')
    C, D = q.shape
    self._ensure(C)
    eps, per_chain = _step_size_tensor(kernel_results.step_size, C, q.device)
    run = run_free(self._handle, q.contiguous().reshape(-1), kernel_results, eps.contiguous(),
                   per_chain, _util.sanitize_seed(seed), first_step, transitions_per_chain,
                   max_leaf_iterations, (C, D))
    self.last_leaf_iterations = run.leaf_iterations
    return run

  def bootstrap_results(self, init_state):
    """nuts.py:456-503 (one gradient evaluation; energy uses unit momenta)."""
    q, layout, is_list = _util.flatten_state(init_state)
    logp, grad = self._target.log_prob_and_grad(q)
    if isinstance(self.step_size, (list, tuple)) and len(self.step_size) != 1:
      raise ValueError('There should be exactly one `step_size` or it should '
                       'have same length as `current_state`.')
    step = _util.as_tensor(self.step_size[0] if isinstance(self.step_size, (list, tuple))
                           else self.step_size, torch.float32, q.device)
    C = q.shape[0]
    return NUTSKernelResults(
        target_log_prob=logp, grads_target_log_prob=_util.unflatten_state(grad, layout, is_list),
        step_size=step, log_accept_ratio=torch.zeros_like(logp),
        leapfrogs_taken=torch.zeros(C, dtype=torch.int32, device=q.device),
        is_accepted=torch.zeros(C, dtype=torch.bool, device=q.device),
        reach_max_depth=torch.zeros(C, dtype=torch.bool, device=q.device),
        has_divergence=torch.zeros(C, dtype=torch.bool, device=q.device),
        energy=logp - 0.5 * q.shape[1], seed=_util.seed_tensor((0, 0)))
