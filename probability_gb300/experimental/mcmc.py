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
  use it as the momentum precision of the next step; with
  num_estimation_steps, stop updating after that many steps."""

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
    return self.inner_kernel.is_calibrated

  @staticmethod
  def _momentum(rv):
    return DiagonalMomentum(rv.variance().to(torch.float32))

  def bootstrap_results(self, init_state):
    inner = self.inner_kernel.bootstrap_results(init_state)
    rv = self.initial_running_variance
    q, _, _ = _util.flatten_state(init_state)
    rv = RunningVariance(*(t.to(q.device) for t in rv))
    if self.num_estimation_steps is None:
      inner = _set_momentum(inner, self._momentum(rv))
    n = -1 if self.num_estimation_steps is None else int(self.num_estimation_steps)
    return DiagonalMassMatrixAdaptationResults(inner_results=inner, running_variance=rv, step=0,
                                               num_estimation_steps=n)

  def one_step(self, current_state, previous_kernel_results, seed=None):
    pkr = previous_kernel_results
    new_state, inner = self.inner_kernel.one_step(current_state, pkr.inner_results, seed=seed)
    step = pkr.step + 1
    rv = pkr.running_variance
    q, _, _ = _util.flatten_state(new_state)
    n_est = pkr.num_estimation_steps
    if n_est < 0 or step <= n_est:
      rv = rv.update(q.to(torch.float64), axis=0)
    if n_est < 0 or step == n_est:
      inner = _set_momentum(inner, self._momentum(rv))
    return new_state, DiagonalMassMatrixAdaptationResults(
        inner_results=inner, running_variance=rv, step=step, num_estimation_steps=n_est)
