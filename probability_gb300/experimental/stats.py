"""RunningVariance (experimental/stats/sample_stats.py RunningVariance):
Welford / Chan running mean and variance, updated with batches."""
import collections

import torch


class RunningVariance(collections.namedtuple('RunningVariance',
                                             ['num_samples', 'mean', 'sum_squared_residuals'])):
  """Streaming variance over samples of a fixed event shape."""
  __slots__ = ()

  @classmethod
  def from_shape(cls, shape=(), dtype=torch.float64, device=None):
    z = torch.zeros(shape, dtype=dtype, device=device)
    return cls(torch.zeros((), dtype=dtype, device=device), z, z.clone())

  @classmethod
  def from_stats(cls, num_samples, mean, variance):
    mean = torch.as_tensor(mean, dtype=torch.float64)
    n = torch.as_tensor(float(num_samples), dtype=torch.float64, device=mean.device)
    return cls(n, mean, torch.as_tensor(variance, dtype=torch.float64, device=mean.device) * n)

  def update(self, new_sample, axis=None):
    """Fold in one sample, or a batch along `axis` (Chan et al.'s merge)."""
    x = torch.as_tensor(new_sample).to(self.mean.dtype)
    if axis is None:
      x = x.unsqueeze(0)
      axis = 0
    m = torch.tensor(float(x.shape[axis]), dtype=self.mean.dtype, device=x.device)
    bmean = x.mean(axis)
    bssr = ((x - bmean.unsqueeze(axis)) ** 2).sum(axis)
    n = self.num_samples + m
    delta = bmean - self.mean
    mean = self.mean + delta * (m / n)
    ssr = self.sum_squared_residuals + bssr + delta * delta * (self.num_samples * m / n)
    return RunningVariance(n, mean, ssr)

  def variance(self, ddof=0):
    return self.sum_squared_residuals / (self.num_samples - ddof)


class RunningPotentialScaleReduction:
  """Streaming potential scale reduction (diagnostic.py:476-568;
  experimental/stats/sample_stats.py:714 RunningPotentialScaleReduction,
  experimental/mcmc/potential_scale_reduction_reducer.py): per-chain running
  means and sums of squared deviations of float32 states [C, ...] are kept
  on the device and updated by the engine (gbm_moments_update), so no draws
  are stored.

  split_chains=True (the potential_scale_reduction option of
  diagnostic.py:517-543) needs the number of draws up front: draws
  0 .. num_draws//2 - 1 and num_draws//2 .. 2 (num_draws//2) - 1 are kept as
  separate half-chains (a trailing odd draw is ignored, as the batch function
  drops it), so after num_draws updates the result equals
  potential_scale_reduction(draws, split_chains=True)."""

  def __init__(self, shape, device=None, split_chains=False, num_draws=None):
    from probability_gb300 import _util
    dev = _util.device() if device is None else torch.device(device)
    self.split = bool(split_chains)
    if self.split and not num_draws:
      raise ValueError('split_chains needs num_draws (the half-chain boundary)')
    self.half = int(num_draws) // 2 if self.split else None
    halves = 2 if self.split else 1
    self._mean = [torch.zeros(shape, dtype=torch.float64, device=dev) for _ in range(halves)]
    self._m2 = [torch.zeros(shape, dtype=torch.float64, device=dev) for _ in range(halves)]
    self.count = 0

  mean = property(lambda self: self._mean[0])
  m2 = property(lambda self: self._m2[0])

  @classmethod
  def from_moments(cls, mean, m2, count):
    r = cls.__new__(cls)
    r.split, r.half = False, None
    r._mean, r._m2, r.count = [mean], [m2], int(count)
    return r

  def update(self, state):
    from probability_gb300 import _native
    x = torch.as_tensor(state, dtype=torch.float32, device=self._mean[0].device).contiguous()
    if x.shape != self._mean[0].shape:
      raise ValueError('state shape %s, expected %s' % (tuple(x.shape),
                                                        tuple(self._mean[0].shape)))
    h, before = 0, self.count
    if self.split:
      if self.count >= 2 * self.half:
        self.count += 1                       # the dropped odd draw
        return self
      h = 1 if self.count >= self.half else 0
      before = self.count - h * self.half
    ctx = _native.Context.current()
    _native.check(_native.lib().gbm_moments_update(
        ctx.handle, _native.ptr(x), x.numel(), before, _native.ptr(self._mean[h]),
        _native.ptr(self._m2[h])), 'gbm_moments_update')
    self.count += 1
    return self

  def potential_scale_reduction(self):
    """R-hat per element: chains (and, split, both halves of every chain)
    along axis 0, by the reference's formula (diagnostic.py:545-567) from the
    running moments."""
    if self.split:
      mean = torch.cat(self._mean, 0)
      m2 = torch.cat(self._m2, 0)
      n = float(self.half)
    else:
      mean, m2, n = self._mean[0], self._m2[0], float(self.count)
    m = float(mean.shape[0])
    w = (m2 / (n - 1.0)).mean(0)                    # mean within-chain variance
    b_div_n = mean.var(0, unbiased=True)            # variance of the chain means
    sigma_2_plus = ((n - 1.0) / n) * w + b_div_n
    return ((m + 1.0) / m) * sigma_2_plus / w - (n - 1.0) / (m * n)


class RunningEffectiveSampleSize:
  """Streaming effective sample size of float32 states [C, ...] (chains on
  axis 0): the engine keeps lagged products up to `max_lag` on the device
  (gbm_autocov_update) instead of the draws, and effective_sample_size()
  evaluates diagnostic.py:203-337 with filter_beyond_lag = max_lag from the
  exact centred autocovariances at lags 0..max_lag -- the value of
  effective_sample_size(draws, filter_beyond_lag=max_lag, ...) on the stored
  draws.  Memory: (3 max_lag + 4) x 4-8 bytes per state element."""

  def __init__(self, shape, max_lag, device=None):
    from probability_gb300 import _util
    dev = _util.device() if device is None else torch.device(device)
    self.shape = tuple(shape)
    self.L = int(max_lag)
    if self.L < 1:
      raise ValueError('max_lag must be >= 1')
    E = 1
    for v in self.shape:
      E *= int(v)
    self.E = E
    self.first = torch.zeros(E, dtype=torch.float32, device=dev)
    self.total = torch.zeros(E, dtype=torch.float64, device=dev)
    self.head = torch.zeros((self.L, E), dtype=torch.float32, device=dev)
    self.ring = torch.zeros((self.L, E), dtype=torch.float32, device=dev)
    self.lag = torch.zeros((self.L + 1, E), dtype=torch.float64, device=dev)
    self.count = 0

  def update(self, state):
    from probability_gb300 import _native
    x = torch.as_tensor(state, dtype=torch.float32, device=self.first.device).contiguous()
    if tuple(x.shape) != self.shape:
      raise ValueError('state shape %s, expected %s' % (tuple(x.shape), self.shape))
    ctx = _native.Context.current()
    P = _native.ptr
    _native.check(_native.lib().gbm_autocov_update(
        ctx.handle, P(x), self.E, self.count, self.L, P(self.first), P(self.total),
        P(self.head), P(self.ring), P(self.lag)), 'gbm_autocov_update')
    self.count += 1
    return self

  def auto_covariance(self):
    """Centred autocovariance [max_lag + 1, *shape] divided by (n - lag), as
    stats/sample_stats.py:44-215 (normalize=False) computes it."""
    n, L = self.count, self.L
    if n <= L:
      raise ValueError('need more than max_lag draws')
    x0 = self.first.to(torch.float64)
    y_head = self.head.to(torch.float64) - x0
    y_ring = self.ring.to(torch.float64) - x0
    m = self.total / n
    prefix = torch.cat([torch.zeros_like(self.total)[None], torch.cumsum(y_head, 0)], 0)
    # Sum of the last k draws, k = 0..L: ring slots (n - 1) % L, (n - 2) % L, ...
    order = [(n - j) % L for j in range(1, L + 1)]
    suffix = torch.cat([torch.zeros_like(self.total)[None],
                        torch.cumsum(y_ring[order], 0)], 0)
    k = torch.arange(L + 1, dtype=torch.float64, device=m.device)[:, None]
    a = self.total - prefix                   # sum_{t >= k} y_t
    b = self.total - suffix                   # sum_{t <= n - 1 - k} y_t
    c = self.lag - m * (a + b) + (n - k) * m * m
    return (c / (n - k)).reshape((L + 1,) + self.shape)

  def effective_sample_size(self, filter_threshold=0., filter_beyond_positive_pairs=False,
                            cross_chain_dims=None):
    """cross_chain_dims as for the batch function on draws [n, C, ...] (1 =
    the chain axis)."""
    from probability_gb300.mcmc.diagnostic import ess_from_auto_covariance
    acov = self.auto_covariance()
    means = None
    if cross_chain_dims is not None:
      means = (self.first.to(torch.float64) + self.total / self.count).reshape(self.shape)
    return ess_from_auto_covariance(acov, self.count, means, filter_threshold,
                                    filter_beyond_positive_pairs, cross_chain_dims)
