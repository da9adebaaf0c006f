"""FP64 log-density + gradient oracle for the three built-in model families.

All functions take a chain-major state ``[C, D]`` and return ``(logp [C],
grad [C, D])`` in float64.  They restate the formulas the reference reaches
through autodiff (internal/util.py:246-308 -> math/gradient.py:28):

* Logistic regression, the inference_gym target
  (spinoffs/inference_gym/inference_gym/targets/logistic_regression.py:88-103)
  with the Bernoulli log-prob of distributions/bernoulli.py:126-140
  (``log p(y) = -softplus(z)(1-y) - softplus(-z) y``) and an iid Normal(0, s)
  prior (distributions/normal.py ``_log_prob``).  The intercept column is a
  column of X supplied by the caller.
* Multivariate normal with a lower-triangular scale, as
  ``MultivariateNormalTriL`` (distributions/mvn_tril.py:44,
  mvn_linear_operator.py:242).
* Non-centred hierarchical normal, the eight-schools pattern of
  mcmc/eight_schools_hmc.py:41-58 with a HalfCauchy scale
  (distributions/half_cauchy.py:138-145) sampled as log(tau) with the
  log-Jacobian added, as TransformedTransitionKernel(Exp) does
  (mcmc/transformed_kernel.py:165).  State layout: [mu, log_tau, z_1..z_J].
"""
import numpy as np

LOG_2PI = np.log(2.0 * np.pi)


def softplus(x):
  return np.logaddexp(0.0, x)


def sigmoid(x):
  return 0.5 * (1.0 + np.tanh(0.5 * x))


def logreg_logp_grad(X, y, beta, prior_scale=1.0):
  X = np.asarray(X, np.float64)
  y = np.asarray(y, np.float64)
  beta = np.asarray(beta, np.float64)
  z = beta @ X.T                                     # [C, N]
  ll = -softplus(z) * (1.0 - y) - softplus(-z) * y   # bernoulli.py:126-140
  s = float(prior_scale)
  prior = -0.5 * (beta / s) ** 2 - np.log(s) - 0.5 * LOG_2PI
  logp = ll.sum(-1) + prior.sum(-1)
  r = y - sigmoid(z)
  grad = r @ X - beta / (s * s)
  return logp, grad


class LogisticRegression:
  def __init__(self, X, y, prior_scale=1.0):
    self.X = np.asarray(X)
    self.y = np.asarray(y)
    self.prior_scale = float(prior_scale)
    self.dim = self.X.shape[1]

  def __call__(self, beta):
    return logreg_logp_grad(self.X, self.y, beta, self.prior_scale)


class MultivariateNormalTriL:
  def __init__(self, loc, scale_tril):
    self.loc = np.asarray(loc, np.float64)
    L = np.asarray(scale_tril, np.float64)
    self.dim = L.shape[-1]
    Linv = np.linalg.inv(L)
    self.precision = Linv.T @ Linv
    self.log_norm = -np.sum(np.log(np.abs(np.diag(L)))) - 0.5 * self.dim * LOG_2PI

  def __call__(self, x):
    dx = np.asarray(x, np.float64) - self.loc
    g = -dx @ self.precision          # precision is symmetric
    logp = 0.5 * np.sum(dx * g, -1) + self.log_norm
    return logp, g


class NonCentredHierarchicalNormal:
  """Eight-schools-like model; state = [mu, log_tau, z_1..z_J]."""

  def __init__(self, y, sigma, mu_scale=5.0, tau_scale=5.0):
    self.y = np.asarray(y, np.float64)
    self.sigma = np.asarray(sigma, np.float64)
    self.mu_scale = float(mu_scale)
    self.tau_scale = float(tau_scale)
    self.dim = self.y.shape[0] + 2

  def __call__(self, x):
    x = np.asarray(x, np.float64)
    mu, eta, z = x[:, 0], x[:, 1], x[:, 2:]
    tau = np.exp(eta)
    sm, st = self.mu_scale, self.tau_scale
    lp_mu = -0.5 * (mu / sm) ** 2 - np.log(sm) - 0.5 * LOG_2PI
    t = tau / st
    lp_tau = np.log(2.0 / np.pi) - np.log(st) - np.log1p(t * t) + eta
    lp_z = np.sum(-0.5 * z * z - 0.5 * LOG_2PI, -1)
    theta = mu[:, None] + tau[:, None] * z
    res = (self.y - theta) / self.sigma
    lp_y = np.sum(-0.5 * res * res - np.log(self.sigma) - 0.5 * LOG_2PI, -1)
    logp = lp_mu + lp_tau + lp_z + lp_y
    r = res / self.sigma                              # d lp_y / d theta
    g = np.empty_like(x)
    g[:, 0] = -mu / (sm * sm) + r.sum(-1)
    g[:, 1] = -2.0 * t * t / (1.0 + t * t) + 1.0 + tau * np.sum(r * z, -1)
    g[:, 2:] = -z + tau[:, None] * r
    return logp, g


class TransformedTarget:
  """A target seen through one elementwise bijector per dimension, the
  transformed log-density TransformedTransitionKernel samples
  (mcmc/transformed_kernel.py:63-95 make_transformed_log_prob with the
  forward maps of bijectors/exp.py, softplus.py, sigmoid.py):
  log p(f(x)) + sum_d log |f_d'(x_d)|.  Codes: 0 identity, 1 exp,
  2 softplus, 3 sigmoid."""

  def __init__(self, inner, codes):
    self.inner = inner
    self.codes = np.asarray(codes, np.int64)
    self.dim = self.codes.shape[0]

  def forward(self, x):
    x = np.asarray(x, np.float64)
    c = self.codes
    return np.where(c == 1, np.exp(x), np.where(c == 2, softplus(x),
                                                np.where(c == 3, sigmoid(x), x)))

  def __call__(self, x):
    x = np.asarray(x, np.float64)
    c = self.codes
    lp, gy = self.inner(self.forward(x))
    s = sigmoid(x)
    # f'(x), log f'(x) and d/dx log f'(x) per bijector
    fp = np.where(c == 1, np.exp(x), np.where(c == 2, s, np.where(c == 3, s * (1 - s), 1.0)))
    logfp = np.where(c == 1, x, np.where(c == 2, -softplus(-x),
                                         np.where(c == 3, -softplus(-x) - softplus(x), 0.0)))
    dlogfp = np.where(c == 1, 1.0, np.where(c == 2, 1.0 - s, np.where(c == 3, 1.0 - 2.0 * s,
                                                                      0.0)))
    return lp + logfp.sum(-1), gy * fp + dlogfp
