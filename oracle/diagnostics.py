"""NumPy restatement of the reference's ESS and R-hat (mcmc/diagnostic.py).

``effective_sample_size`` follows diagnostic.py:203-337 with the FFT
autocovariance of stats/sample_stats.py:44-215 (centred, zero-padded to a
power of two >= 2n, divided by n - lag).  ``potential_scale_reduction``
follows diagnostic.py:476-568 (Brooks-Gelman with optional split chains).
States are ``[n_draws, chains, ...]``.
"""
import numpy as np


def auto_covariance(x, axis=0):
  """stats/sample_stats.py:44-215 with normalize=False."""
  x = np.moveaxis(np.asarray(x, np.float64), axis, -1)
  x = x - x.mean(-1, keepdims=True)
  n = x.shape[-1]
  size = int(2 ** np.ceil(np.log2(2 * n)))
  f = np.fft.rfft(x, n=size, axis=-1)
  r = np.fft.irfft(f * np.conj(f), n=size, axis=-1)[..., :n]
  r = r / (n - np.arange(n))
  return np.moveaxis(r, -1, axis)


def effective_sample_size(states, filter_threshold=0.0, filter_beyond_lag=None,
                          filter_beyond_positive_pairs=False,
                          cross_chain_dims=None):
  """diagnostic.py:203-337.  With cross_chain_dims=None the result has the
  chain axis (sum it for a total ESS, as nuts_test.py:398-399 does).
  filter_beyond_lag keeps lags 0..filter_beyond_lag of the autocorrelation
  (the max_lags of auto_correlation, diagnostic.py:254-258)."""
  states = np.asarray(states, np.float64)
  n = states.shape[0]
  acov = auto_covariance(states, 0)
  if filter_beyond_lag is not None:
    acov = acov[:int(filter_beyond_lag) + 1]
  if cross_chain_dims is not None:
    ax = cross_chain_dims
    num_chains = states.shape[ax]
    between = np.var(states.mean(0), axis=ax - 1, ddof=1)
    within = np.mean(acov[0], axis=ax - 1)
    approx = within + between
    mean_acov = np.mean(acov, axis=ax)
    rho = 1.0 - (within - mean_acov) / approx
  else:
    rho = acov / acov[:1]
    num_chains = 1
  k = np.arange(rho.shape[0], dtype=np.float64)
  nk = ((n - k) / n).reshape((-1,) + (1,) * (rho.ndim - 1))
  weighted = nk * rho
  if filter_beyond_positive_pairs:
    m = rho.shape[0] - rho.shape[0] % 2
    pair = lambda v: v[:m].reshape((m // 2, 2) + v.shape[1:]).sum(1)
    mask = (pair(rho) < 0).astype(np.float64)
    mask = np.maximum(1.0 - np.cumsum(mask, 0), 0.0)
    weighted = pair(weighted) * mask
  elif filter_threshold is not None:
    mask = (rho < filter_threshold).astype(np.float64)
    mask = np.maximum(1.0 - np.cumsum(mask, 0), 0.0)
    weighted = weighted * mask
  return num_chains * n / (-1.0 + 2.0 * weighted.sum(0))


def potential_scale_reduction(chains_states, independent_chain_ndims=1,
                              split_chains=False):
  """diagnostic.py:476-568."""
  s = np.asarray(chains_states, np.float64)
  if split_chains:
    n = s.shape[0] - s.shape[0] % 2
    s = s[:n].reshape((2, n // 2) + s.shape[1:])
    s = np.moveaxis(s, 0, 1)
    independent_chain_ndims += 1
  chain_axes = tuple(range(1, 1 + independent_chain_ndims))
  all_axes = (0,) + chain_axes
  n = s.shape[0]
  m = np.prod([s.shape[a] for a in chain_axes])
  b_div_n = np.var(s.mean(0, keepdims=True), axis=all_axes, ddof=1)
  w = np.mean(np.var(s, axis=0, keepdims=True, ddof=1), axis=all_axes)
  sigma_2_plus = ((n - 1) / n) * w + b_div_n
  return ((m + 1.0) / m) * sigma_2_plus / w - (n - 1.0) / (m * n)
