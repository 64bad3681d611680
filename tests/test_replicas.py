"""bench.py's multi-rank path (replicas only): two gloo ranks on the CPU
agree on the max of their timings and the sum of their body-steps."""
from __future__ import annotations

import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch
    import torch.distributed as dist
    import bench
    import datetime
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=60))
    dev = torch.device("cpu")
    t = bench.dist_max(10.0 + rank, world, dev)
    n = bench.dist_sum(100.0 * (rank + 1), world, dev)
    out[rank] = (t, n)
    dist.destroy_process_group()


def test_two_replicas_reduce():
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    assert res[0] == res[1] == (11.0, 300.0)
