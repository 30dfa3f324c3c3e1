"""Multi-GPU is replicas only: every rank steps its own copy of the
workload, and bench.py reports the slowest rank's time and the particle-steps
of all ranks over it.  Two gloo ranks on the CPU check that aggregation."""
from __future__ import annotations

import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, q):
    import sys
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms, value = bench.aggregate_replicas(ms=100.0 + 50.0 * rank, n_active=1000 * (rank + 1), steps=10, dist=dist)
    q.put((rank, ms, value))
    dist.destroy_process_group()


def test_two_replicas_aggregate_max_time_and_total_work():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
    for rank, ms, value in res:
        assert ms == 150.0                                       # the slowest rank
        assert abs(value - (1000 + 2000) * 10 / 0.150) < 1e-6   # all ranks' work over it
