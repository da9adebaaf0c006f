"""TransitionKernel contract (mcmc/kernel.py:27-164 of the reference)."""
import abc
import collections


class TransitionKernel(abc.ABC):
  """Base class: ``one_step``, ``bootstrap_results``, ``is_calibrated``,
  ``parameters``, ``copy`` -- the reference's plugin interface
  (mcmc/kernel.py:86-164)."""

  @abc.abstractmethod
  def one_step(self, current_state, previous_kernel_results, seed=None):
    """Returns (next_state, kernel_results)."""

  @abc.abstractmethod
  def bootstrap_results(self, init_state):
    """Returns initial kernel results for ``init_state``."""

  @property
  def is_calibrated(self):
    return True

  @property
  def parameters(self):
    return self._parameters

  def copy(self, **override_parameter_kwargs):
    """mcmc/kernel.py:148-164: a new kernel with some parameters replaced."""
    params = dict(self.parameters)
    params.update(override_parameter_kwargs)
    return type(self)(**params)

  @property
  def experimental_shard_axis_names(self):
    return self._parameters.get('experimental_shard_axis_names')

  def experimental_with_shard_axes(self, shard_axis_names):
    if shard_axis_names:
      raise NotImplementedError('the engine runs on one GPU; state sharding is not supported')
    return self.copy(experimental_shard_axis_names=shard_axis_names)


class PrettyNamedTupleMixin:
  """Readable repr for results namedtuples (mcmc/internal/util.py)."""
  __slots__ = ()

  def __repr__(self):
    return '{}(\n{}\n)'.format(
        type(self).__name__,
        ',\n'.join('  {}={}'.format(k, repr(v).replace('\n', '\n    '))
                   for k, v in self._asdict().items()))


def results_type(name, fields):
  base = collections.namedtuple(name, fields)
  return type(name, (PrettyNamedTupleMixin, base), {'__slots__': ()})
