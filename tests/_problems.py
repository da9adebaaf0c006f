"""Seeded synthetic problems shared by the tests (shapes follow the
workloads the engine is measured on, scaled down where the oracle must
finish in seconds)."""
import numpy as np


def logreg_data(n, d, seed=0, scale=1.0, intercept=True):
  """X [n, d] with column 0 = 1 and iid N(0, scale^2) elsewhere; true beta
  ~ N(0, I); y ~ Bernoulli(sigmoid(X beta))."""
  rng = np.random.default_rng(seed)
  X = rng.normal(size=(n, d)) * scale
  if intercept:
    X[:, 0] = 1.0
  beta = rng.normal(size=d)
  z = X @ beta
  y = (rng.uniform(size=n) < 1.0 / (1.0 + np.exp(-z))).astype(np.float32)
  return X.astype(np.float32), y, beta


def init_state(chains, d, seed=0, scale=0.1):
  rng = np.random.default_rng(seed + 1000)
  return (rng.normal(size=(chains, d)) * scale).astype(np.float32)
