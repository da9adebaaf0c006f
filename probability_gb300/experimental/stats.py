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
  """Streaming potential scale reduction (diagnostic.py:476-568 without split
  chains; experimental/mcmc/potential_scale_reduction_reducer.py): per-chain
  running means and sums of squared deviations of float32 states [C, ...]
  are kept on the device and updated by the engine (gbm_moments_update), so
  no draws are stored."""

  def __init__(self, shape, device=None):
    from probability_gb300 import _util
    dev = _util.device() if device is None else torch.device(device)
    self.mean = torch.zeros(shape, dtype=torch.float64, device=dev)
    self.m2 = torch.zeros(shape, dtype=torch.float64, device=dev)
    self.count = 0

  @classmethod
  def from_moments(cls, mean, m2, count):
    r = cls.__new__(cls)
    r.mean, r.m2, r.count = mean, m2, int(count)
    return r

  def update(self, state):
    from probability_gb300 import _native
    x = torch.as_tensor(state, dtype=torch.float32, device=self.mean.device).contiguous()
    if x.shape != self.mean.shape:
      raise ValueError('state shape %s, expected %s' % (tuple(x.shape), tuple(self.mean.shape)))
    ctx = _native.Context.current()
    _native.check(_native.lib().gbm_moments_update(
        ctx.handle, _native.ptr(x), x.numel(), self.count, _native.ptr(self.mean),
        _native.ptr(self.m2)), 'gbm_moments_update')
    self.count += 1
    return self

  def potential_scale_reduction(self):
    """R-hat per element: chains along axis 0 (the reference's formula,
    diagnostic.py:545-567, from the running moments)."""
    n, m = float(self.count), float(self.mean.shape[0])
    w = (self.m2 / (n - 1.0)).mean(0)                    # mean within-chain variance
    b_div_n = self.mean.var(0, unbiased=True)            # variance of the chain means
    sigma_2_plus = ((n - 1.0) / n) * w + b_div_n
    return ((m + 1.0) / m) * sigma_2_plus / w - (n - 1.0) / (m * n)
