"""The multi-GPU path of the bench: replicas, one process per GPU, no
data-path collective; the job's throughput is every rank's particle-steps over
the slowest rank's time.  Two gloo ranks on the host exercise the reduction
and the barrier the bench runs under torchrun."""
from __future__ import annotations

import importlib
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, queue) -> None:
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sys.path.insert(0, ROOT)
        bench = importlib.import_module("bench")
        assert bench.WORLD == world
        bench._barrier()
        # rank r: (r + 1) x 1000 particle-steps in (r + 1) x 100 ms
        value, slowest = bench.whole_job(100.0 * (rank + 1), 1000 * (rank + 1))
        queue.put((rank, value, slowest))
    finally:
        dist.destroy_process_group()


def test_two_replicas_aggregate_over_the_slowest_rank():
    pytest.importorskip("torch.distributed")
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, queue)) for r in range(world)]
    for p in procs:
        p.start()
    results = sorted(queue.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, value, slowest in results:
        assert slowest == pytest.approx(200.0)
        assert value == pytest.approx(3000 / 0.2)
