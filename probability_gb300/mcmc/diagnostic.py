"""Effective sample size and R-hat (reference: mcmc/diagnostic.py).

Measurement utilities, not part of the sampling path: they run with torch
tensor ops on whatever device the draws are on.  ESS follows
diagnostic.py:203-337 with the FFT autocovariance of
stats/sample_stats.py:44-215; R-hat follows diagnostic.py:476-568.
States are ``[n_draws, chains, ...]``.
"""
import math

import torch


def _auto_covariance(x):
  """Centred autocovariance along axis 0, divided by (n - lag)."""
  x = x.to(torch.float64)
  x = x - x.mean(0, keepdim=True)
  n = x.shape[0]
  size = 2 ** int(math.ceil(math.log2(2 * n)))
  f = torch.fft.rfft(x, n=size, dim=0)
  r = torch.fft.irfft(f * f.conj(), n=size, dim=0)[:n]
  denom = (n - torch.arange(n, dtype=torch.float64, device=x.device))
  return r / denom.reshape((-1,) + (1,) * (x.dim() - 1))


def effective_sample_size(states, filter_threshold=0., filter_beyond_lag=None,
                          filter_beyond_positive_pairs=False, cross_chain_dims=None):
  """diagnostic.py:203-337; filter_beyond_lag truncates the autocorrelation
  at that lag (auto_correlation's max_lags, :254-258)."""
  states = torch.as_tensor(states)
  n = states.shape[0]
  acov = _auto_covariance(states)
  if filter_beyond_lag is not None:
    acov = acov[:int(filter_beyond_lag) + 1]
  means = states.to(torch.float64).mean(0) if cross_chain_dims is not None else None
  return ess_from_auto_covariance(acov, n, means, filter_threshold,
                                  filter_beyond_positive_pairs, cross_chain_dims)


def ess_from_auto_covariance(acov, n, chain_means=None, filter_threshold=0.,
                             filter_beyond_positive_pairs=False, cross_chain_dims=None):
  """The ESS formula of diagnostic.py:242-337 from centred autocovariances
  acov [lags, ...] of n-draw chains (divided by n - lag); with
  cross_chain_dims (an axis of the draws, so axis cross_chain_dims - 1 of
  acov[k]) the chain means give the between-chain variance."""
  if cross_chain_dims is not None:
    ax = int(cross_chain_dims)
    num_chains = acov.shape[ax]
    between = chain_means.var(dim=ax - 1, unbiased=True)
    within = acov[0].mean(dim=ax - 1)
    approx = within + between
    rho = 1.0 - (within - acov.mean(dim=ax)) / approx
  else:
    rho = acov / acov[:1]
    num_chains = 1
  k = torch.arange(rho.shape[0], dtype=torch.float64, device=rho.device)
  nk = ((n - k) / n).reshape((-1,) + (1,) * (rho.dim() - 1))
  weighted = nk * rho
  if filter_beyond_positive_pairs:
    m = rho.shape[0] - rho.shape[0] % 2
    pair = lambda v: v[:m].reshape((m // 2, 2) + tuple(v.shape[1:])).sum(1)
    mask = (pair(rho) < 0).to(torch.float64)
    mask = torch.clamp(1.0 - torch.cumsum(mask, 0), min=0.0)
    weighted = pair(weighted) * mask
  elif filter_threshold is not None:
    mask = (rho < filter_threshold).to(torch.float64)
    mask = torch.clamp(1.0 - torch.cumsum(mask, 0), min=0.0)
    weighted = weighted * mask
  return num_chains * n / (-1.0 + 2.0 * weighted.sum(0))


def potential_scale_reduction(chains_states, independent_chain_ndims=1, split_chains=False):
  s = torch.as_tensor(chains_states).to(torch.float64)
  if split_chains:
    n = s.shape[0] - s.shape[0] % 2
    s = s[:n].reshape((2, n // 2) + tuple(s.shape[1:])).movedim(0, 1)
    independent_chain_ndims += 1
  chain_axes = tuple(range(1, 1 + independent_chain_ndims))
  all_axes = (0,) + chain_axes
  n = s.shape[0]
  m = 1
  for a in chain_axes:
    m *= s.shape[a]
  b_div_n = s.mean(0, keepdim=True).var(dim=all_axes, unbiased=True)
  w = s.var(dim=0, keepdim=True, unbiased=True).mean(dim=all_axes)
  sigma_2_plus = ((n - 1) / n) * w + b_div_n
  return ((m + 1.0) / m) * sigma_2_plus / w - (n - 1.0) / (m * n)
