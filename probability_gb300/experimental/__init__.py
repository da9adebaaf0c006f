"""Drop-in subset of ``tfp.experimental`` backed by the engine."""
from probability_gb300.experimental import mcmc, stats

__all__ = ['mcmc', 'stats']
