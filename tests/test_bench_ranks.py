"""bench.py's replica mode on CPU: two gloo ranks combine their units (sum)
and times (maximum), as N GPUs under torchrun do with NCCL."""
from __future__ import annotations

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, out):
    os.environ.update(WORLD_SIZE=str(world), RANK=str(rank), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import bench
    r = bench.Ranks()
    r.init("gloo")
    r.barrier()
    rays = 1000.0 * (rank + 1)
    ms = 5.0 + rank
    out.put((rank, r.reduce(rays, "sum"), r.reduce(ms, "max")))
    r.close()


def test_two_replicas_combine_units_and_times():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(i, world, port, q)) for i in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, total, tmax in res:
        assert total == 3000.0 and tmax == 6.0


def test_single_process_needs_no_group():
    import bench
    r = bench.Ranks()
    r.init("gloo")   # WORLD_SIZE unset: no process group
    assert r.reduce(7.0, "sum") == 7.0 and r.reduce(3.0, "max") == 3.0
    r.barrier()
    r.close()
