"""Drop-in subset of ``tfp.mcmc`` backed by the GB300 engine."""
from probability_gb300.mcmc.diagnostic import effective_sample_size, potential_scale_reduction
from probability_gb300.mcmc.dual_averaging_step_size_adaptation import (
    DualAveragingStepSizeAdaptation, DualAveragingStepSizeAdaptationResults,
    reduce_log_harmonic_mean_exp, reduce_logmeanexp)
from probability_gb300.mcmc.hmc import (HamiltonianMonteCarlo, UncalibratedHamiltonianMonteCarlo,
                                        UncalibratedHamiltonianMonteCarloKernelResults)
from probability_gb300.mcmc.kernel import TransitionKernel
from probability_gb300.mcmc.metropolis_hastings import (MetropolisHastings,
                                                        MetropolisHastingsKernelResults)
from probability_gb300.mcmc.nuts import NoUTurnSampler, NUTSKernelResults
from probability_gb300.mcmc.sample import (ChainRun, CheckpointableStatesAndTrace,
                                           StatesAndTrace, run_chain, sample_chain)
from probability_gb300.mcmc.transformed_kernel import (TransformedTransitionKernel,
                                                       TransformedTransitionKernelResults)
from probability_gb300.mcmc.simple_step_size_adaptation import (
    hmc_like_log_accept_prob_getter_fn, hmc_like_step_size_getter_fn,
    hmc_like_step_size_setter_fn)

__all__ = [
    'ChainRun', 'run_chain', 'CheckpointableStatesAndTrace', 'DualAveragingStepSizeAdaptation',
    'DualAveragingStepSizeAdaptationResults', 'HamiltonianMonteCarlo',
    'MetropolisHastings', 'MetropolisHastingsKernelResults', 'NUTSKernelResults', 'NoUTurnSampler', 'StatesAndTrace',
    'TransformedTransitionKernel', 'TransformedTransitionKernelResults',
    'TransitionKernel', 'UncalibratedHamiltonianMonteCarlo',
    'UncalibratedHamiltonianMonteCarloKernelResults', 'effective_sample_size',
    'hmc_like_log_accept_prob_getter_fn', 'hmc_like_step_size_getter_fn',
    'hmc_like_step_size_setter_fn', 'potential_scale_reduction', 'reduce_log_harmonic_mean_exp',
    'reduce_logmeanexp', 'sample_chain',
]
