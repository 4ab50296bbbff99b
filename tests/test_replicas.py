"""The N > 1 path: replicas with a max-over-ranks time and a sum of units, on 2 gloo ranks (CPU)."""
from __future__ import annotations

import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import torch.distributed as dist

    from voxelyze_gb300.replicas import aggregate_rate, barrier

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    barrier()
    rate, units, secs = aggregate_rate(local_units=1000 * (rank + 1), local_seconds=1.0 + rank)
    out[rank] = (rate, units, secs)
    dist.destroy_process_group()


def test_two_rank_aggregation():
    import torch.multiprocessing as mp

    world = 2
    mgr = mp.Manager()
    out = mgr.dict()
    mp.start_processes(_worker, args=(world, _free_port(), out), nprocs=world, start_method="spawn")
    for r in range(world):
        rate, units, secs = out[r]
        assert units == 3000.0
        assert secs == 2.0
        assert rate == 1500.0


def test_single_process_fallback():
    from voxelyze_gb300.replicas import aggregate_rate

    assert aggregate_rate(500, 2.0) == (250.0, 500.0, 2.0)
