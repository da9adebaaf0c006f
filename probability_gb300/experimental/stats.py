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
