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


def laplace(X, y, prior_scale=1.0, iters=50):
  """MAP and Hessian H = X^T diag(s(1-s)) X + I/prior_scale^2 of the
  logistic-regression posterior (float64 Newton iterations)."""
  X = np.asarray(X, np.float64)
  y = np.asarray(y, np.float64)
  D = X.shape[1]
  prec = 1.0 / prior_scale ** 2
  beta = np.zeros(D)
  for _ in range(iters):
    s = 1.0 / (1.0 + np.exp(-(X @ beta)))
    H = (X * (s * (1 - s))[:, None]).T @ X + prec * np.eye(D)
    step = np.linalg.solve(H, X.T @ (y - s) - prec * beta)
    beta = beta + step
    if np.abs(step).max() < 1e-13:
      break
  s = 1.0 / (1.0 + np.exp(-(X @ beta)))
  H = (X * (s * (1 - s))[:, None]).T @ X + prec * np.eye(D)
  return beta, H


def logreg_posterior_moments(X, y, n=200000, seed=0, prior_scale=1.0):
  """Posterior mean and variance of each coefficient by self-normalised
  importance sampling in float64 (proposal: the Laplace approximation with
  its covariance inflated 1.5^2), with the standard errors of both
  estimates: the ground truth of the long-run moment tests."""
  X = np.asarray(X, np.float64)
  y = np.asarray(y, np.float64)
  mode, H = laplace(X, y, prior_scale)
  L = np.linalg.cholesky(np.linalg.inv(H)) * 1.5
  rng = np.random.default_rng(seed)
  z = rng.standard_normal((n, X.shape[1]))
  b = mode + z @ L.T
  logq = -0.5 * np.sum(z * z, 1)
  eta = b @ X.T
  loglik = (y * eta - np.logaddexp(0.0, eta)).sum(1)
  logp = loglik - 0.5 * np.sum(b * b, 1) / prior_scale ** 2
  lw = logp - logq
  w = np.exp(lw - lw.max())
  w /= w.sum()
  mean = w @ b
  var = w @ (b - mean) ** 2
  mean_se = np.sqrt(np.sum(w[:, None] ** 2 * (b - mean) ** 2, 0))
  var_se = np.sqrt(np.sum(w[:, None] ** 2 * ((b - mean) ** 2 - var) ** 2, 0))
  return mean, var, mean_se, var_se
