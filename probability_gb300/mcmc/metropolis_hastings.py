"""MetropolisHastings results (reference: mcmc/metropolis_hastings.py:41-56).

The accept/reject step itself is fused into the engine's HMC transition
(``gbm_hmc_one_step``); this module keeps the results structure so nested
accessors such as ``kr.accepted_results.step_size`` behave as in the
reference.
"""
from probability_gb300.mcmc import kernel as kernel_base

MetropolisHastingsKernelResults = kernel_base.results_type(
    'MetropolisHastingsKernelResults',
    ['accepted_results', 'is_accepted', 'log_accept_ratio', 'proposed_state',
     'proposed_results', 'extra', 'seed'])


def has_target_log_prob(kernel_results):
  """metropolis_hastings.py:291-293."""
  return getattr(kernel_results, 'target_log_prob', None) is not None
