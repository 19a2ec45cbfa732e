"""Diagnostics of a population sharded over several processes (one GPU each).

Particles are independent within an interval, so a run shards by particle:
each rank pushes, injects and splits its own particles with no exchange on
the data path.  Only the driver's diagnostics see the whole population, and
these functions form them from the ranks' local ones with torch.distributed
(NCCL between GPUs, gloo on the host):

* the momentum histogram (src/main.cpp:1907-1964): an all-reduce sum of the
  bins.  The weights are dyadic (0.5^level), so the sums are exact in any
  order and the global histogram equals the one of the whole population;
* the summary row (src/main.cpp:1845-1901): counts and weight sums added,
  minima and maxima reduced, averages from the ranks' sums (the reference
  sums serially; the combination differs from it by rounding only);
* global particle ids: an exclusive scan of the ranks' stored counts, so
  rank r's local index i is global index offset_r + i (the order of the ranks'
  stores concatenated);
* the per-rank share of a frame's injection (the driver injects
  particles_per_frame x rank_scale per frame, src/main.cpp:2325-2327).

The reference has no distributed run (its only MPI user is an external
Fortran comparator); this is the exchange its particle sharding would need.
"""
from __future__ import annotations

from typing import Dict, Optional

import numpy as np

SUMMARY_SUM_KEYS = ("stored", "active", "inactive", "weight_sum")


def _dist():
    import torch.distributed as dist
    if not dist.is_initialized():
        raise RuntimeError("sharded diagnostics need an initialised torch.distributed group")
    return dist


def _device(dist, group=None) -> str:
    if dist.get_backend(group) == "nccl":
        import torch
        return f"cuda:{torch.cuda.current_device()}"
    return "cpu"


def _all_reduce(values: np.ndarray, op: str, group=None) -> np.ndarray:
    import torch
    dist = _dist()
    t = torch.tensor(np.asarray(values, dtype=np.float64), device=_device(dist, group))
    ops = {"sum": dist.ReduceOp.SUM, "min": dist.ReduceOp.MIN, "max": dist.ReduceOp.MAX}
    dist.all_reduce(t, op=ops[op], group=group)
    return t.cpu().numpy()


def reduce_histogram(bins: np.ndarray, group=None) -> np.ndarray:
    """The whole population's weight histogram from the ranks' local ones."""
    return _all_reduce(bins, "sum", group)


def reduce_summary(local: Dict[str, float], group=None) -> Dict[str, float]:
    """The whole population's summary row from the ranks' kpt_summary
    dictionaries (stored, active, inactive, weight_sum, p_min/max/avg,
    dt_min/max/avg, max_split_level).  Ranks with no active particle do not
    contribute to the minima, maxima and averages."""
    active = float(local["active"])
    sums = _all_reduce([float(local[k]) for k in SUMMARY_SUM_KEYS] +
                       [local["p_avg"] * active, local["dt_avg"] * active], "sum", group)
    inf = float("inf")
    mins = _all_reduce([local["p_min"] if active else inf, local["dt_min"] if active else inf],
                       "min", group)
    maxs = _all_reduce([local["p_max"] if active else -inf,
                        local["dt_max"] if active else -inf,
                        float(local["max_split_level"])], "max", group)
    out = {k: (int(round(v)) if k != "weight_sum" else float(v))
           for k, v in zip(SUMMARY_SUM_KEYS, sums[:4])}
    total_active = out["active"]
    out["max_split_level"] = int(maxs[2])
    if total_active > 0:
        out.update(p_min=float(mins[0]), p_max=float(maxs[0]), dt_min=float(mins[1]),
                   dt_max=float(maxs[1]), p_avg=float(sums[4] / total_active),
                   dt_avg=float(sums[5] / total_active))
    else:
        out.update(p_min=0.0, p_max=0.0, dt_min=0.0, dt_max=0.0, p_avg=0.0, dt_avg=0.0)
    return out


def global_offset(count: int, group=None) -> int:
    """Exclusive scan of the ranks' stored counts: the global index of this
    rank's first particle."""
    import torch
    dist = _dist()
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    local = torch.tensor([int(count)], dtype=torch.int64, device=_device(dist, group))
    counts = [torch.zeros_like(local) for _ in range(world)]
    dist.all_gather(counts, local, group=group)
    return int(sum(int(c.item()) for c in counts[:rank]))


def injection_share(requested: int, rank: Optional[int] = None, world: Optional[int] = None,
                    group=None) -> int:
    """This rank's share of a frame's `requested` injections: an even split,
    the first requested % world ranks taking one more."""
    if rank is None or world is None:
        dist = _dist()
        rank, world = dist.get_rank(group), dist.get_world_size(group)
    return requested // world + (1 if rank < requested % world else 0)
