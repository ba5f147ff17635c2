"""The multi-rank path of bench.py on CPU: two gloo ranks (replicas), the job time is the max
over ranks and the value counts the units of every rank."""
import os
import sys
from pathlib import Path

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parent.parent


def _rank(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    sys.path.insert(0, str(ROOT))
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = 100.0 * (rank + 1)  # rank 1 is the slower one
    t_max, value = bench.combine_ranks(dist, ms, world, n_units=1000, steps=2, device="cpu")
    q.put((rank, t_max, value))
    dist.destroy_process_group()


def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + (os.getpid() % 1000)
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    out = sorted(q.get(timeout=10) for _ in range(2))
    for rank, t_max, value in out:
        assert t_max == 200.0
        assert value == pytest.approx(2 * 1000 * 2 / 0.2)
