"""Tensor exchange and seed helpers for the host-side kernel classes."""
import ctypes
import random

import numpy as np
import torch

from probability_gb300 import _native


def device():
  if not torch.cuda.is_available():
    raise RuntimeError('the gb300 MCMC engine needs a CUDA device; none is available')
  return torch.device('cuda', torch.cuda.current_device())


def as_tensor(x, dtype=None, dev=None):
  """Import any array (torch, DLPack producer such as TF/JAX, NumPy, Python
  scalars/lists) as a contiguous torch tensor on the engine's device."""
  dev = dev or device()
  if isinstance(x, torch.Tensor):
    t = x
  elif hasattr(x, '__dlpack__') and not isinstance(x, np.ndarray):
    t = torch.from_dlpack(x)
  else:
    t = torch.as_tensor(np.asarray(x))
  if dtype is not None and t.dtype != dtype:
    t = t.to(dtype)
  return t.to(dev).contiguous()


def flatten_state(state):
  """List-of-parts state -> ([C, D] tensor, part sizes, is_list).

  The engine works on one chain-major part; multi-part states are
  concatenated along the event axis and split back on output."""
  if isinstance(state, (list, tuple)):
    parts = [as_tensor(s, torch.float32) for s in state]
    c = parts[0].shape[0]
    flat = [p.reshape(c, -1) for p in parts]
    sizes = [f.shape[1] for f in flat]
    shapes = [p.shape for p in parts]
    return torch.cat(flat, 1).contiguous(), (sizes, shapes), True
  t = as_tensor(state, torch.float32)
  if t.dim() == 1:
    return t.reshape(-1, 1).contiguous(), ([1], [t.shape]), False
  return t.reshape(t.shape[0], -1).contiguous(), ([t[0].numel()], [t.shape]), False


def unflatten_state(flat, layout, is_list):
  sizes, shapes = layout
  parts = torch.split(flat, sizes, dim=1)
  parts = [p.reshape(s) for p, s in zip(parts, shapes)]
  return list(parts) if is_list else parts[0]


def sanitize_seed(seed):
  """int / (int, int) / tensor / None -> (uint32, uint32).

  None draws a fresh key from Python's RNG (the reference's stateful-seed
  path, internal/samplers.py:79-133)."""
  if seed is None:
    return (random.getrandbits(32), random.getrandbits(32))
  if isinstance(seed, torch.Tensor):
    seed = seed.detach().cpu().numpy()
  if isinstance(seed, (int, np.integer)):
    s = int(seed) & 0xFFFFFFFFFFFFFFFF
    return (s & 0xFFFFFFFF, (s >> 32) & 0xFFFFFFFF)
  arr = np.asarray(seed).reshape(-1)
  if arr.size != 2:
    raise ValueError('seed must be an int or a pair of ints, got shape %s' % (arr.shape,))
  return (int(arr[0]) & 0xFFFFFFFF, int(arr[1]) & 0xFFFFFFFF)


def step_key(seed, step):
  out = (ctypes.c_uint32 * 2)()
  _native.check(_native.lib().gbm_step_key(_native.seed_words(seed), int(step), out),
                'gbm_step_key')
  return (int(out[0]), int(out[1]))


def seed_tensor(seed):
  return torch.tensor([seed[0], seed[1]], dtype=torch.int64)
