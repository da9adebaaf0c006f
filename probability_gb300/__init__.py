"""GB300-native gradient-MCMC engine: a drop-in for tfp.mcmc's
HamiltonianMonteCarlo, NoUTurnSampler, DualAveragingStepSizeAdaptation and
sample_chain, with hand-written sm_103a kernels behind a C ABI
(include/gb300_mcmc.h)."""
from probability_gb300 import bijectors, experimental, mcmc, targets
from probability_gb300.batch import BatchedNoUTurnSampler, TargetBatch
from probability_gb300.targets import (LogisticRegression, MultivariateNormalTriL,
                                       NonCentredHierarchicalNormal)

__all__ = ['bijectors', 'experimental', 'mcmc', 'targets', 'LogisticRegression', 'MultivariateNormalTriL',
           'NonCentredHierarchicalNormal', 'TargetBatch', 'BatchedNoUTurnSampler']
