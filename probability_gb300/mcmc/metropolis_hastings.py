"""MetropolisHastings on the engine (reference: mcmc/metropolis_hastings.py).

``MetropolisHastings(inner_kernel)`` wraps any engine kernel whose results
carry ``target_log_prob`` (and, for a non-symmetric proposal,
``log_acceptance_correction``) -- in practice the engine's
``UncalibratedHamiltonianMonteCarlo``.  The accept/reject of
metropolis_hastings.py:160-254 runs on the device
(``gbm_metropolis_hastings_step``): log_accept_ratio = safe_sum(proposed -
current + correction), accept iff log U < log_accept_ratio, per-chain select
of the state; the per-chain select of the nested results (``choose``,
mcmc/internal/util.py:103-164) is a device-side ``where``.  The uniform U is
the transition key's Metropolis-Hastings draw, the same one the fused
``HamiltonianMonteCarlo`` uses, so
``MetropolisHastings(UncalibratedHamiltonianMonteCarlo(...))`` and
``HamiltonianMonteCarlo(...)`` give identical results for the same seed.
"""
import warnings

import torch

from probability_gb300 import _native, _util
from probability_gb300.mcmc import kernel as kernel_base

MetropolisHastingsKernelResults = kernel_base.results_type(
    'MetropolisHastingsKernelResults',
    ['accepted_results', 'is_accepted', 'log_accept_ratio', 'proposed_state',
     'proposed_results', 'extra', 'seed'])


def has_target_log_prob(kernel_results):
  """metropolis_hastings.py:291-293."""
  return getattr(kernel_results, 'target_log_prob', None) is not None


def choose(is_accepted, proposed, current):
  """mcmc/internal/util.py:103-164: per-chain select over a results tuple
  (tensors whose leading dimension is the chain axis, lists of them, nested
  results); anything else is taken from `proposed`."""
  def pick(p, c):
    if isinstance(p, torch.Tensor) and isinstance(c, torch.Tensor) and p.shape == c.shape \
        and p.dim() >= 1 and p.shape[0] == is_accepted.shape[0]:
      m = is_accepted.reshape((-1,) + (1,) * (p.dim() - 1))
      return torch.where(m, p, c)
    if isinstance(p, list) and isinstance(c, list) and len(p) == len(c) and p:
      return [pick(a, b) for a, b in zip(p, c)]
    if hasattr(p, '_fields') and hasattr(c, '_fields') and type(p) is type(c):
      return type(p)(*[pick(a, b) for a, b in zip(p, c)])
    return p
  return pick(proposed, current)


class MetropolisHastings(kernel_base.TransitionKernel):
  """metropolis_hastings.py:59-297: calibrates an uncalibrated proposal."""

  def __init__(self, inner_kernel, name=None):
    if inner_kernel.is_calibrated:
      warnings.warn('Supplied `TransitionKernel` is already calibrated. '
                    'Composing `MetropolisHastings` `TransitionKernel` '
                    'may not be required.')
    self._parameters = dict(inner_kernel=inner_kernel, name=name)

  inner_kernel = property(lambda self: self._parameters['inner_kernel'])
  name = property(lambda self: self._parameters['name'])

  @property
  def is_calibrated(self):
    return True

  def one_step(self, current_state, previous_kernel_results, seed=None):
    """metropolis_hastings.py:160-254."""
    seed = _util.sanitize_seed(seed)
    pkr = previous_kernel_results
    proposed_state, proposed_results = self.inner_kernel.one_step(
        current_state, pkr.accepted_results, seed=seed)
    if not has_target_log_prob(proposed_results):
      raise ValueError('"proposed_results" must have a "target_log_prob" member.')
    if not has_target_log_prob(pkr.accepted_results):
      raise ValueError('"previous_kernel_results.accepted_results" must have a '
                       '"target_log_prob" member.')
    corr = getattr(proposed_results, 'log_acceptance_correction', None)
    if corr is None:
      warnings.warn('Supplied inner `TransitionKernel` does not have a '
                    '`log_acceptance_correction`. Assuming its value is `0.`')
    q, layout, is_list = _util.flatten_state(current_state)
    qp, _, _ = _util.flatten_state(proposed_state)
    C, D = q.shape
    dev = q.device
    f64 = lambda t: _util.as_tensor(t, torch.float64, dev).reshape(C).contiguous()
    cur = f64(pkr.accepted_results.target_log_prob)
    prop = f64(proposed_results.target_log_prob)
    cor = None if corr is None else f64(corr)
    q, qp = q.contiguous(), qp.contiguous()
    nq = torch.empty_like(q)
    lar = torch.empty(C, dtype=torch.float64, device=dev)
    acc = torch.empty(C, dtype=torch.uint8, device=dev)
    ctx = _native.Context.current()
    P = _native.ptr
    _native.check(_native.lib().gbm_metropolis_hastings_step(
        ctx.handle, C, D, _native.seed_words(seed), P(cur), P(prop), P(cor), P(q), P(qp),
        P(nq), P(lar), P(acc)), 'gbm_metropolis_hastings_step')
    is_accepted = acc.bool()
    accepted = choose(is_accepted, proposed_results, pkr.accepted_results)
    kr = MetropolisHastingsKernelResults(
        accepted_results=accepted, is_accepted=is_accepted, log_accept_ratio=lar,
        proposed_state=proposed_state, proposed_results=proposed_results, extra=[],
        seed=_util.seed_tensor(seed))
    return _util.unflatten_state(nq, layout, is_list), kr

  def bootstrap_results(self, init_state):
    """metropolis_hastings.py:256-288."""
    pkr = self.inner_kernel.bootstrap_results(init_state)
    if not has_target_log_prob(pkr):
      raise ValueError('"target_log_prob" must be a member of '
                       '`inner_kernel` results.')
    x = _util.as_tensor(pkr.target_log_prob, torch.float64)
    return MetropolisHastingsKernelResults(
        accepted_results=pkr, is_accepted=torch.ones_like(x, dtype=torch.bool),
        log_accept_ratio=torch.zeros_like(x), proposed_state=init_state, proposed_results=pkr,
        extra=[], seed=_util.seed_tensor((0, 0)))
