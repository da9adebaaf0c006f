"""PreconditionedNoUTurnSampler and DiagonalMassMatrixAdaptation on the
engine (reference: experimental/mcmc/preconditioned_nuts.py:169,
diagonal_mass_matrix_adaptation.py:73).

The momentum distribution is diagonal: precision diag(v) with v the running
variance of the state (preconditioning_utils.py:40-97), i.e. the inverse
mass matrix.  The engine's NUTS kernels take v directly
(gbm_nuts_set_inverse_mass): momentum z / sqrt(v), drift by the velocity
v * p, kinetic energy 1/2 sum v p^2, U-turn checks against velocities.
"""
import collections

import torch

from probability_gb300 import _native, _util
from probability_gb300.experimental.stats import RunningVariance
from probability_gb300.mcmc import kernel as kernel_base
from probability_gb300.mcmc.nuts import NoUTurnSampler

PreconditionedNUTSKernelResults = kernel_base.results_type('PreconditionedNUTSKernelResults', [
    'target_log_prob', 'grads_target_log_prob', 'step_size', 'log_accept_ratio',
    'leapfrogs_taken', 'is_accepted', 'reach_max_depth', 'has_divergence', 'energy',
    'momentum_distribution', 'seed'])

DiagonalMassMatrixAdaptationResults = kernel_base.results_type(
    'DiagonalMassMatrixAdaptationResults',
    ['inner_results', 'running_variance', 'step', 'num_estimation_steps'])


class DiagonalMomentum(collections.namedtuple('DiagonalMomentum', ['precision_diag'])):
  """Momentum distribution N(0, diag(1 / precision_diag)): the
  MultivariateNormalPrecisionFactorLinearOperator of
  preconditioning_utils.py:82-88 with a diagonal precision (the running
  variance of the state, float32 [D] on the device)."""
  __slots__ = ()

  def variance(self):
    """Variance of the momentum, 1 / precision_diag."""
    return 1.0 / self.precision_diag


class PreconditionedNoUTurnSampler(NoUTurnSampler):
  """experimental/mcmc/preconditioned_nuts.py:169-457."""

  def __init__(self, target_log_prob_fn, step_size, max_tree_depth=10, max_energy_diff=1000.,
               unrolled_leapfrog_steps=1, parallel_iterations=10, momentum_distribution=None,
               experimental_shard_axis_names=None, name=None):
    super().__init__(target_log_prob_fn, step_size, max_tree_depth, max_energy_diff,
                     unrolled_leapfrog_steps, parallel_iterations,
                     experimental_shard_axis_names, name)
    self._parameters['momentum_distribution'] = momentum_distribution

  momentum_distribution = property(lambda self: self._parameters['momentum_distribution'])

  def _momentum(self, dim, dev):
    md = self.momentum_distribution
    if md is None:
      return DiagonalMomentum(torch.ones(dim, dtype=torch.float32, device=dev))
    if not isinstance(md, DiagonalMomentum):
      md = DiagonalMomentum(_util.as_tensor(md, torch.float32, dev).reshape(-1))
    return md

  def bootstrap_results(self, init_state):
    kr = super().bootstrap_results(init_state)
    q, _, _ = _util.flatten_state(init_state)
    return PreconditionedNUTSKernelResults(
        *kr[:9], momentum_distribution=self._momentum(q.shape[1], q.device), seed=kr.seed)

  def one_step(self, current_state, previous_kernel_results, seed=None):
    pkr = previous_kernel_results
    q, _, _ = _util.flatten_state(current_state)
    self._ensure(q.shape[0])
    v = _util.as_tensor(pkr.momentum_distribution.precision_diag, torch.float32,
                        q.device).contiguous()
    if v.numel() != q.shape[1]:
      raise ValueError('momentum precision must have one entry per state dimension')
    self._inv_mass = v                     # kept alive while the engine reads it
    _native.check(_native.lib().gbm_nuts_set_inverse_mass(self._handle, _native.ptr(v), 0),
                  'gbm_nuts_set_inverse_mass')
    nq, kr = super().one_step(current_state, pkr, seed=seed)
    return nq, PreconditionedNUTSKernelResults(
        *kr[:9], momentum_distribution=pkr.momentum_distribution, seed=kr.seed)


def _set_momentum(results, momentum):
  if hasattr(results, 'momentum_distribution'):
    return results._replace(momentum_distribution=momentum)
  if hasattr(results, 'inner_results'):
    return results._replace(inner_results=_set_momentum(results.inner_results, momentum))
  raise ValueError('no inner results carry a momentum_distribution')


class DiagonalMassMatrixAdaptation(kernel_base.TransitionKernel):
  """experimental/mcmc/diagonal_mass_matrix_adaptation.py:73-340: after each
  step, fold the new state (every chain a sample) into a running variance and
  use it as the momentum precision of the next step.  With
  num_estimation_steps given, the variance is updated while step <=
  results.num_estimation_steps and the momentum set once, when step ==
  results.num_estimation_steps (a results value of -1 therefore skips
  adaptation, which WindowedAdaptation uses in its first fast window)."""

  def __init__(self, inner_kernel, initial_running_variance, num_estimation_steps=None,
               name=None):
    self._parameters = dict(inner_kernel=inner_kernel,
                            initial_running_variance=initial_running_variance,
                            num_estimation_steps=num_estimation_steps, name=name)

  inner_kernel = property(lambda self: self._parameters['inner_kernel'])
  initial_running_variance = property(lambda self: self._parameters['initial_running_variance'])
  num_estimation_steps = property(lambda self: self._parameters['num_estimation_steps'])

  @property
  def is_calibrated(self):
    if self.num_estimation_steps is None:          # :335-339
      return False
    return self.inner_kernel.is_calibrated

  @staticmethod
  def _momentum(rv):
    return DiagonalMomentum(rv.variance().to(torch.float32))

  def _bootstrap_from_inner_results(self, init_state, inner_results):
    """:318-331: fresh running variance, step 0."""
    q, _, _ = _util.flatten_state(init_state)
    rv = RunningVariance(*(t.to(q.device) for t in self.initial_running_variance))
    n = -1 if self.num_estimation_steps is None else int(self.num_estimation_steps)
    return DiagonalMassMatrixAdaptationResults(inner_results=inner_results, running_variance=rv,
                                               step=0, num_estimation_steps=n)

  def bootstrap_results(self, init_state):
    results = self._bootstrap_from_inner_results(
        init_state, self.inner_kernel.bootstrap_results(init_state))
    if self.num_estimation_steps is not None:
      return results        # the momentum is set at the end of estimation (:290-292)
    return results._replace(
        inner_results=_set_momentum(results.inner_results, self._momentum(
            results.running_variance)))

  def one_step(self, current_state, previous_kernel_results, seed=None):
    """:190-278."""
    pkr = previous_kernel_results
    new_state, inner = self.inner_kernel.one_step(current_state, pkr.inner_results, seed=seed)
    step = pkr.step + 1
    rv = pkr.running_variance
    q, _, _ = _util.flatten_state(new_state)
    n_est = pkr.num_estimation_steps
    always = self.num_estimation_steps is None
    if always or step <= n_est:
      rv = rv.update(q.to(torch.float64), axis=0)
    if always or step == n_est:
      inner = _set_momentum(inner, self._momentum(rv))
    return new_state, DiagonalMassMatrixAdaptationResults(
        inner_results=inner, running_variance=rv, step=step, num_estimation_steps=n_est)


# ---------------------------------------------------------------------------
# Windowed adaptation (experimental/mcmc/windowed_sampling.py)
# ---------------------------------------------------------------------------
WindowedAdaptationResults = kernel_base.results_type('WindowedAdaptationResults',
                                                     ['inner_results', 'step'])


def _get_window_sizes(num_adaptation_steps):
  """windowed_sampling.py:322-347: a first fast window of 3/20, slow windows
  of 1, 2, 4 and 8 twentieths, and a last fast window with the rest."""
  slow = num_adaptation_steps // 20
  first = 3 * slow
  last = num_adaptation_steps - 15 * slow - first
  return first, slow, last


class WindowedAdaptation(kernel_base.TransitionKernel):
  """windowed_sampling.py:366-517 around
  DiagonalMassMatrixAdaptation(DualAveragingStepSizeAdaptation(...)): the
  step size adapts in every window; the diagonal mass matrix is estimated
  afresh in each slow window and installed at its end; dual averaging
  restarts at each slow window and at the last fast window."""

  def __init__(self, inner_kernel, num_adaptation_steps, name=None):
    self._parameters = dict(inner_kernel=inner_kernel,
                            num_adaptation_steps=num_adaptation_steps, name=name)

  inner_kernel = property(lambda self: self._parameters['inner_kernel'])
  num_adaptation_steps = property(lambda self: self._parameters['num_adaptation_steps'])
  name = property(lambda self: self._parameters['name'])

  @property
  def is_calibrated(self):
    return self.inner_kernel.is_calibrated

  def bootstrap_results(self, init_state):
    return WindowedAdaptationResults(inner_results=self.inner_kernel.bootstrap_results(init_state),
                                     step=0)

  def _reset_dual_averaging(self, current_state, dmma_results, num_adaptation_steps):
    da = self.inner_kernel.inner_kernel
    da_results = dmma_results.inner_results
    inner = da.step_size_setter_fn(da_results.inner_results, da_results.new_step_size)
    fresh = da._bootstrap_from_inner_results(current_state, inner)
    return fresh._replace(num_adaptation_steps=int(num_adaptation_steps))

  def one_step(self, current_state, previous_kernel_results, seed=None):
    """windowed_sampling.py:419-498."""
    pkr = previous_kernel_results
    prev = pkr.inner_results                      # DiagonalMassMatrixAdaptationResults
    step = int(pkr.step)
    first, slow, last = _get_window_sizes(int(self.num_adaptation_steps))
    slow_starts = [first + slow * (2 ** i - 1) for i in range(1, 4)]
    if step == 0:                                 # first fast window: no mass matrix
      prev = prev._replace(
          inner_results=prev.inner_results._replace(num_adaptation_steps=first + slow),
          num_estimation_steps=-1)
    elif step == first:                           # first slow window: start estimating
      prev = prev._replace(step=0, num_estimation_steps=slow)
    elif step in slow_starts:                     # later slow windows: restart both
      size = step - first + slow
      dmma = self.inner_kernel._bootstrap_from_inner_results(current_state, prev.inner_results)
      prev = dmma._replace(inner_results=self._reset_dual_averaging(current_state, dmma, size),
                           num_estimation_steps=size)
    elif step == first + 15 * slow:               # last fast window: restart dual averaging
      prev = prev._replace(inner_results=self._reset_dual_averaging(current_state, prev, last))
    new_state, new_inner = self.inner_kernel.one_step(current_state, prev, seed=seed)
    return new_state, pkr._replace(inner_results=new_inner, step=step + 1)


def default_nuts_trace_fn(state, bijector, is_adapting, pkr):
  """windowed_sampling.py:63-103: sampler statistics of each draw."""
  from probability_gb300.mcmc.simple_step_size_adaptation import get_innermost
  del state, bijector
  energy_diff = get_innermost(pkr, 'log_accept_ratio')
  return {
      'step_size': get_innermost(pkr, 'step_size'),
      'tune': is_adapting,
      'target_log_prob': get_innermost(pkr, 'target_log_prob'),
      'diverging': get_innermost(pkr, 'has_divergence'),
      'accept_ratio': torch.clamp(torch.exp(energy_diff), max=1.0),
      'variance_scaling': get_innermost(pkr, 'momentum_distribution').variance(),
      'n_steps': get_innermost(pkr, 'leapfrogs_taken'),
      'is_accepted': get_innermost(pkr, 'is_accepted')}


def windowed_adaptive_nuts(n_draws, target, *, n_chains=64, num_adaptation_steps=500,
                           current_state=None, init_step_size=None, dual_averaging_kwargs=None,
                           max_tree_depth=10, max_energy_diff=500., unrolled_leapfrog_steps=1,
                           parallel_iterations=10, trace_fn=default_nuts_trace_fn,
                           return_final_kernel_results=False, discard_tuning=True,
                           chain_axis_names=None, seed=None):
  """windowed_sampling.py:603-729 for one of the engine's targets.

  The reference samples a pinned JointDistribution in its unconstrained
  space; the engine takes the target directly (a built-in family, or a
  TransformedTarget for constrained parameters), whose state is that space.
  Same schedule: WindowedAdaptation(DiagonalMassMatrixAdaptation(
  DualAveragingStepSizeAdaptation(PreconditionedNoUTurnSampler))) with a
  target accept probability of 0.85 and the harmonic-mean reduction of the
  accept probabilities by default; chains start uniformly in (-2, 2) and the
  step size at 0.5 D^-1/4 (windowed_sampling.py:566-589) unless given.
  Returns the draws (and the trace, and final kernel results) as the
  reference does.
  """
  from probability_gb300 import targets as targets_mod
  from probability_gb300.mcmc.dual_averaging_step_size_adaptation import (
      DualAveragingStepSizeAdaptation, reduce_log_harmonic_mean_exp)
  from probability_gb300.mcmc.sample import (CheckpointableStatesAndTrace, StatesAndTrace,
                                             sample_chain)
  if chain_axis_names:
    raise NotImplementedError('the engine runs on one GPU; chains are not sharded')
  tgt = targets_mod.resolve(target)
  dim = tgt.dim
  dev = _util.device()
  if current_state is None:
    gen = torch.Generator(device='cpu')
    gen.manual_seed(int(_util.sanitize_seed(seed)[0]))
    current_state = (torch.rand((int(n_chains), dim), generator=gen, dtype=torch.float32)
                     * 4.0 - 2.0).to(dev)
  q, _, _ = _util.flatten_state(current_state)
  step_size = init_step_size if init_step_size is not None else 0.5 * float(q.shape[1]) ** -0.25
  da_kwargs = dict(dual_averaging_kwargs or {})
  da_kwargs.setdefault('target_accept_prob', 0.85)
  da_kwargs.setdefault('reduce_fn', reduce_log_harmonic_mean_exp)
  da_kwargs['num_adaptation_steps'] = int(num_adaptation_steps)
  nuts = PreconditionedNoUTurnSampler(
      tgt, step_size=step_size, max_tree_depth=max_tree_depth, max_energy_diff=max_energy_diff,
      unrolled_leapfrog_steps=unrolled_leapfrog_steps, parallel_iterations=parallel_iterations,
      momentum_distribution=DiagonalMomentum(torch.ones(q.shape[1], dtype=torch.float32,
                                                        device=q.device)))
  rv = RunningVariance.from_stats(0, torch.zeros(q.shape[1], device=q.device),
                                  torch.ones(q.shape[1], device=q.device))
  kernel = WindowedAdaptation(
      DiagonalMassMatrixAdaptation(DualAveragingStepSizeAdaptation(nuts, **da_kwargs),
                                   initial_running_variance=rv,
                                   num_estimation_steps=int(num_adaptation_steps)),
      num_adaptation_steps=int(num_adaptation_steps))
  no_trace = trace_fn is None
  tfn = (lambda *a: ()) if no_trace else trace_fn
  n_adapt = int(num_adaptation_steps)
  ret = sample_chain(
      int(n_draws) if discard_tuning else int(n_draws) + n_adapt, q, kernel=kernel,
      num_burnin_steps=n_adapt if discard_tuning else 0,
      trace_fn=lambda state, pkr: tfn(state, None, pkr.step <= n_adapt,
                                      pkr.inner_results.inner_results.inner_results),
      return_final_kernel_results=return_final_kernel_results, seed=seed)
  if return_final_kernel_results:
    return CheckpointableStatesAndTrace(all_states=ret.all_states, trace=ret.trace,
                                        final_kernel_results=ret.final_kernel_results)
  if no_trace:
    return ret.all_states
  return StatesAndTrace(all_states=ret.all_states, trace=ret.trace)
