"""CPU oracle for the gradient-MCMC hot path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product package imports this
directory; only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may use it, and
only to check the engine's results (or as the timed CPU restatement of the
reference).

It is a NumPy restatement of TensorFlow Probability's ``tfp.mcmc`` algorithms
(HamiltonianMonteCarlo, MetropolisHastings, SimpleLeapfrogIntegrator,
NoUTurnSampler, DualAveragingStepSizeAdaptation, sample_chain, the ESS and
R-hat diagnostics) and of the log-density formulas of the three built-in
model families.  Each function cites the reference file:line it follows
(paths relative to the tensorflow_probability project root).

Random draws: the reference draws from TensorFlow's stateless RNG, whose bits
are not reproducible without TensorFlow.  The oracle instead consumes draws
from ``oracle.philox`` -- a NumPy mirror of the engine's own counter-based
Philox4x32-10 stream, addressed by (transition key, draw kind, tree depth,
leaf, element) -- so the engine and the oracle are fed identical momentum,
direction and uniform draws.  Parity against the reference's own RNG bits is
therefore unpinned; the algorithmic parity is pinned by the reference's golden
vectors (NUTS instruction tables, dual-averaging constants, NaN rejection).
"""
