"""Replica path of `bench.py --gpus N` (independent chain replicas, one per
process) on CPU: two gloo ranks combine throughput as total work over the
slowest replica and gather draws into one chain population."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip('torch')
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
  s = socket.socket()
  s.bind(('127.0.0.1', 0))
  port = s.getsockname()[1]
  s.close()
  return port


def _worker(rank, world, port, out):
  os.environ['MASTER_ADDR'] = '127.0.0.1'
  os.environ['MASTER_PORT'] = str(port)
  dist.init_process_group('gloo', rank=rank, world_size=world)
  from probability_gb300 import replicas
  secs, units = replicas.combine_throughput(1.0 + rank, 100 * (rank + 1))
  draws = torch.full((5, 3, 2), float(rank))
  allc = replicas.gather_draws(draws)
  init = replicas.replica_init((4, 2), seed=7, rank=rank)
  out.put((rank, secs, units, tuple(allc.shape), float(allc[:, 3:].mean()),
           replicas.replica_key((7, 0), rank), init.tolist()))
  dist.barrier()
  dist.destroy_process_group()


def test_two_replicas_combine_on_gloo():
  ctx = mp.get_context('spawn')
  q = ctx.Queue()
  port = _free_port()
  procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
  for p in procs:
    p.start()
  res = sorted(q.get(timeout=120) for _ in procs)
  for p in procs:
    p.join(timeout=60)
    assert p.exitcode == 0
  for rank, secs, units, shape, tail_mean, key, init in res:
    assert secs == 2.0                  # the slowest replica's time
    assert units == 300                 # total work
    assert shape == (5, 6, 2)           # chains of both replicas
    assert tail_mean == 1.0             # rank 1's chains follow rank 0's
  assert res[0][5] != res[1][5]         # distinct keys per replica
  assert not np.allclose(res[0][6], res[1][6])


def test_combine_without_process_group_is_local():
  from probability_gb300 import replicas
  assert replicas.combine_throughput(2.5, 10) == (2.5, 10)
