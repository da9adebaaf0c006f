"""Step-size getter/setter helpers (mcmc/simple_step_size_adaptation.py:32-61)."""
import torch


def _innermost_holder(kernel_results, name):
  """Walk .inner_results / .accepted_results to the innermost results that
  have ``name`` (internal/unnest.py:147-221)."""
  chain = [kernel_results]
  r = kernel_results
  while True:
    nxt = None
    for f in ('inner_results', 'accepted_results'):
      if hasattr(r, f):
        cand = getattr(r, f)
        if hasattr(cand, '_fields'):
          nxt = cand
          break
    if nxt is None:
      break
    chain.append(nxt)
    r = nxt
  for r in reversed(chain):
    if name in getattr(r, '_fields', ()):
      return chain, r
  raise AttributeError('no results field named %r' % name)


def get_innermost(kernel_results, name):
  return getattr(_innermost_holder(kernel_results, name)[1], name)


def replace_innermost(kernel_results, **kw):
  """internal/unnest.py:221: replace the innermost occurrence of each field."""
  name = next(iter(kw))
  chain, holder = _innermost_holder(kernel_results, name)
  idx = chain.index(holder)
  new = holder._replace(**kw)
  for parent in reversed(chain[:idx]):
    for f in ('inner_results', 'accepted_results'):
      if hasattr(parent, f) and getattr(parent, f) is chain[chain.index(parent) + 1]:
        new = parent._replace(**{f: new})
        break
  return new


def hmc_like_step_size_setter_fn(kernel_results, new_step_size):
  return replace_innermost(kernel_results, step_size=new_step_size)


def hmc_like_step_size_getter_fn(kernel_results):
  return get_innermost(kernel_results, 'step_size')


def hmc_like_log_accept_prob_getter_fn(kernel_results):
  """min(log_accept_ratio, 0) with non-finite -> -inf."""
  lar = get_innermost(kernel_results, 'log_accept_ratio')
  safe = torch.where(torch.isfinite(lar), lar, torch.full_like(lar, -float('inf')))
  return torch.clamp(safe, max=0.0)
