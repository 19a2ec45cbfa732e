"""The sharded path's diagnostics exchange on two and three gloo ranks.

A population (momenta log-uniform, split levels 0-6 with dyadic weights,
statuses mixed) is split over the ranks by the injection share; each rank
forms its local 128-bin histogram and summary with the oracle, and
kokkos-particletransport_gb300/sharded.py combines them.  Against the oracle
on the whole population: histogram bins bit for bit, counts, weight sum,
minima, maxima and split level exact, averages within 1e-13; the exclusive
scan of the stored counts gives every rank the global index of its first
particle.  One case leaves a rank with no active particle.
"""
from __future__ import annotations

import importlib
import multiprocessing as mp
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _population(n: int, seed: int, dead_tail: int):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    binding = importlib.import_module("binding")
    rng = np.random.default_rng(seed)
    parts = binding.empty_particles(n)
    parts["p"][:] = np.exp(rng.uniform(np.log(5e-3), np.log(2e1), n))
    parts["dt"][:] = rng.uniform(1e-6, 1e-3, n)
    parts["level"][:] = rng.integers(0, 7, n).astype(np.int32)
    parts["w"][:] = 0.5 ** parts["level"]
    parts["status"][:] = rng.choice([0, 0, 0, 1, 2], n).astype(np.int32)
    if dead_tail:
        parts["status"][n - dead_tail:] = 1  # the last rank's particles all escaped
    return binding, parts


def _rank(rank, world, port, n, dead_tail, queue):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sys.path.insert(0, ROOT)
        sharded = importlib.import_module("kokkos-particletransport_gb300.sharded")
        binding, parts = _population(n, 7, dead_tail)
        oracle = binding.Oracle()
        shares = [sharded.injection_share(n, r, world) for r in range(world)]
        assert sharded.injection_share(n) == shares[rank]
        first = sum(shares[:rank])
        local = {k: np.ascontiguousarray(v[first:first + shares[rank]]) for k, v in parts.items()}
        count = shares[rank]
        bins = sharded.reduce_histogram(oracle.histogram(1e-2, 1e1, 128, count, local))
        summary = sharded.reduce_summary(oracle.summarize(count, local))
        offset = sharded.global_offset(count)
        queue.put((rank, bins, summary, offset, first))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world,n,dead_tail", [(2, 50_001, 0), (3, 30_000, 10_000)])
def test_sharded_diagnostics_equal_the_whole_populations(world, n, dead_tail):
    pytest.importorskip("torch.distributed")
    port = _free_port()
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, n, dead_tail, queue))
             for r in range(world)]
    for p in procs:
        p.start()
    results = sorted((queue.get(timeout=180) for _ in range(world)), key=lambda t: t[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    binding, parts = _population(n, 7, dead_tail)
    oracle = binding.Oracle()
    want_bins = oracle.histogram(1e-2, 1e1, 128, n, parts)
    want = oracle.summarize(n, parts)
    for rank, bins, summary, offset, first in results:
        assert np.array_equal(bins, want_bins), rank
        for key in ("stored", "active", "inactive", "max_split_level", "weight_sum", "p_min",
                    "p_max", "dt_min", "dt_max"):
            assert summary[key] == want[key], (rank, key)
        for key in ("p_avg", "dt_avg"):
            assert summary[key] == pytest.approx(want[key], rel=1e-13), (rank, key)
        assert offset == first
