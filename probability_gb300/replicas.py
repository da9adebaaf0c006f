"""Independent chain replicas across processes (one GPU each).

Chains are independent, so several GPUs run separate replicas of a sampler
with their own initial states and keys; nothing is exchanged while they
sample (the reference's only cross-chain coupling, dual averaging's mean
accept probability, dual_averaging_step_size_adaptation.py:419-435, stays
per replica).  After a run, throughput combines as total work over the
slowest replica's time, and cross-replica diagnostics treat the replicas'
chains as one population.
"""
import numpy as np
import torch


def replica_key(seed, rank):
  """Key of replica `rank` for a run seeded with `seed` (int or pair)."""
  s = seed if isinstance(seed, (tuple, list)) else (int(seed), 0)
  return (int(s[0]) & 0xFFFFFFFF, (int(s[1]) + 0x9E3779B9 * int(rank)) & 0xFFFFFFFF)


def replica_init(shape, seed, rank, scale=0.1):
  """Seeded N(0, scale^2) initial state of replica `rank` (float32)."""
  rng = np.random.default_rng([int(seed), int(rank)])
  return (rng.normal(size=shape) * scale).astype(np.float32)


def combine_throughput(seconds, units, group=None):
  """(max seconds over replicas, total units over replicas) through
  torch.distributed (any backend), or the local values without a group."""
  import torch.distributed as dist
  if not (dist.is_available() and dist.is_initialized()):
    return float(seconds), int(units)
  dev = torch.device('cuda', torch.cuda.current_device()) \
      if dist.get_backend(group) == 'nccl' else torch.device('cpu')
  t = torch.tensor([float(seconds)], dtype=torch.float64, device=dev)
  u = torch.tensor([int(units)], dtype=torch.int64, device=dev)
  dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
  dist.all_reduce(u, op=dist.ReduceOp.SUM, group=group)
  return float(t.item()), int(u.item())


def gather_draws(draws, group=None):
  """Concatenate every replica's draws [n, C, D] along the chain axis (for
  cross-replica ESS and R-hat); returns the local draws without a group."""
  import torch.distributed as dist
  if not (dist.is_available() and dist.is_initialized()):
    return draws
  out = [torch.empty_like(draws) for _ in range(dist.get_world_size(group))]
  dist.all_gather(out, draws.contiguous(), group=group)
  return torch.cat(out, dim=1)
