"""Batched runs: many independent runs pushed by one launch per interval.

Every run of a batch must end bitwise where the same run pushed on its own
with kpt_push_interval ends (same seed, frames and cell sort), whatever the
batch composition, the schedule chosen by the autotuner, or whether the
interval loop is replayed from a CUDA graph.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NAMES = ("x", "y", "p", "t", "dt", "w", "mu", "status", "level")


def _runs(kpt, fields_mod, binding, oracle, focused):
    """Five runs of different grids, settings, sizes, seeds and start frames."""
    specs = [(32, 64, False, 300, 0.05, 11, 3), (64, 128, True, 2500, 0.05, 12, 5),
             (48, 96, False, 1200, 0.2, 13, 0), (16, 32, True, 90, 0.05, 14, 9),
             (64, 64, False, 4000, 0.01, 15, 2)]
    runs = []
    for k, (nx, ny, stretched, n, ratio, seed, frame) in enumerate(specs):
        ye = fields_mod.stretched_edges(ny, -2.0, 2.0) if stretched else None
        f0 = fields_mod.harris_field(nx, ny, y_edges=ye, island_amplitude=0.05 * k,
                                     sheet_width=0.05 + 0.03 * k, noise=0.01, seed=seed)
        f1 = fields_mod.harris_field(nx, ny, y_edges=ye, island_amplitude=0.05 * k,
                                     sheet_width=0.05 + 0.03 * k, noise=0.01, seed=seed + 100)
        params = binding.default_params(kperp_over_kpara=ratio, focused=int(focused))
        if k == 2:
            params.update(dt_min_rel=1e-2, dt_max_rel=1e-2)
        grid = oracle.grid(f0.x_edges, f0.y_edges)
        start = binding.empty_particles(n)
        count = oracle.inject(grid, params, frame * 0.1, frame, seed, n, 0, n, start)
        oracle.free_grid(grid)
        runs.append(dict(f0=f0, f1=f1, settings=kpt.settings_from_dict(params), seed=seed,
                         frame=frame, start=start, count=count))
    return runs


def _tables(ctx, kpt, run, focused):
    kind = kpt.TABLE_FOCUSED21 if focused else kpt.TABLE_PARKER16
    return (ctx.field(run["f0"], kind, kpt.PRECISION_MIXED),
            ctx.field(run["f1"], kind, kpt.PRECISION_MIXED))


@pytest.mark.parametrize("focused", [False, True])
@pytest.mark.parametrize("use_graph", [True, False])
def test_batch_equals_runs_pushed_one_by_one(ctx, kpt, fields_mod, binding, oracle, focused,
                                             use_graph):
    intervals, tile = 3, 8
    runs = _runs(kpt, fields_mod, binding, oracle, focused)
    # one by one
    singles, single_stats = [], []
    for run in runs:
        lower, upper = _tables(ctx, kpt, run, focused)
        parts = ctx.particles(run["count"])
        parts.upload(run["start"], run["count"])
        for k in range(intervals):
            ctx.sort(parts, lower, tile, tile)
            stats = ctx.push_interval(parts, lower, upper, run["settings"], run["frame"] + k,
                                      run["seed"])
        singles.append(parts.download())
        single_stats.append(stats)
        for h in (parts, lower, upper):
            h.close()
    # batched
    batch = ctx.batch()
    handles = []
    for run in runs:
        lower, upper = _tables(ctx, kpt, run, focused)
        parts = ctx.particles(run["count"])
        parts.upload(run["start"], run["count"])
        batch.add_run(parts, lower, upper, run["settings"], run["seed"], run["frame"])
        handles.append((parts, lower, upper))
    batch.set_schedule(sort_tile=tile, blocks_per_sm=0, sort_every=1)
    batch.run(intervals, use_graph=use_graph)
    for r, (run, (parts, _, _)) in enumerate(zip(runs, handles)):
        got = parts.download()
        for name in NAMES:
            assert np.array_equal(got[name], singles[r][name]), (r, name)
        st = batch.stats(r)
        assert st.particle_steps == single_stats[r].particle_steps
        assert st.pushed == single_stats[r].pushed
        assert batch.frame(r) == run["frame"] + intervals
    batch.close()
    for hs in handles:
        for h in hs:
            h.close()


@pytest.mark.parametrize("focused", [False, True])
def test_launch_shapes_give_identical_results(ctx, kpt, fields_mod, binding, oracle, focused):
    """Block size and particles per lane change only the schedule: every
    shape ends bit for bit where the default one does."""
    runs = _runs(kpt, fields_mod, binding, oracle, focused)
    results = {}
    for shape in ((128, 1), (64, 1), (256, 1), (64, 2), (128, 2), (256, 2)):
        batch = ctx.batch()
        handles = []
        for run in runs:
            lower, upper = _tables(ctx, kpt, run, focused)
            parts = ctx.particles(run["count"])
            parts.upload(run["start"], run["count"])
            batch.add_run(parts, lower, upper, run["settings"], run["seed"], run["frame"])
            handles.append((parts, lower, upper))
        batch.set_schedule(sort_tile=8, blocks_per_sm=0, sort_every=1)
        batch.set_launch_shape(*shape)
        batch.run(2)
        results[shape] = [h[0].download() for h in handles]
        steps = [batch.stats(r).particle_steps for r in range(len(runs))]
        if shape == (128, 1):
            base_steps = steps
        assert steps == base_steps, shape
        batch.close()
        for hs in handles:
            for h in hs:
                h.close()
    for shape, got in results.items():
        for r in range(len(runs)):
            for name in NAMES:
                assert np.array_equal(got[r][name], results[(128, 1)][r][name]), (shape, r, name)
    with pytest.raises(kpt.KptError, match="threads_per_block"):
        batch = ctx.batch()
        try:
            batch.set_launch_shape(96, 1)
        finally:
            batch.close()


def test_autotune_keeps_state_and_results(ctx, kpt, fields_mod, binding, oracle):
    runs = _runs(kpt, fields_mod, binding, oracle, False)
    batch = ctx.batch()
    handles = []
    for run in runs:
        lower, upper = _tables(ctx, kpt, run, False)
        parts = ctx.particles(run["count"])
        parts.upload(run["start"], run["count"])
        batch.add_run(parts, lower, upper, run["settings"], run["seed"], run["frame"])
        handles.append((parts, lower, upper))
    before = [h[0].download() for h in handles]
    tuning = batch.autotune(1)
    # stage 1: 7 sort schedules; stage 2: 3 block shapes x 2 particles per
    # lane x 3 residencies, less the default already timed
    assert tuning["candidates"] == 7 + 17 and tuning["best_ms"] > 0
    assert tuning["repeats"] == 3 and tuning["spread"] >= 0.0
    assert tuning["threads_per_block"] in (64, 128, 256)
    assert tuning["particles_per_lane"] in (1, 2)
    sched = batch.schedule()
    assert sched["sort_tile"] == tuning["sort_tile"]
    assert batch.launch_shape() == {"threads_per_block": tuning["threads_per_block"],
                                    "particles_per_lane": tuning["particles_per_lane"]}
    for r, (parts, _, _) in enumerate(handles):
        after = parts.download()
        for name in NAMES:
            assert np.array_equal(after[name], before[r][name]), (r, name)
        assert batch.frame(r) == runs[r]["frame"]
    # the tuned schedule gives the same particles as the default one
    batch.run(2)
    tuned = [h[0].download() for h in handles]
    for r, (parts, _, _) in enumerate(handles):
        parts.upload(before[r], runs[r]["count"])
    batch2 = ctx.batch()
    for r, run in enumerate(runs):
        parts, lower, upper = handles[r]
        batch2.add_run(parts, lower, upper, run["settings"], run["seed"], run["frame"])
    batch2.set_schedule(sort_tile=0)
    batch2.run(2, use_graph=False)
    for r, (parts, _, _) in enumerate(handles):
        got = parts.download()
        for name in NAMES:
            assert np.array_equal(got[name], tuned[r][name]), (r, name)
    batch.close()
    batch2.close()
    for hs in handles:
        for h in hs:
            h.close()


def test_batch_rejects_mixed_models_and_fp64(ctx, kpt, fields_mod, binding):
    f = fields_mod.harris_field(16, 32, noise=0.0, seed=1)
    parts = ctx.particles(8)
    batch = ctx.batch()
    parker = kpt.settings_from_dict(binding.default_params())
    focused = kpt.settings_from_dict(binding.default_params(focused=1))
    lo64 = ctx.field(f, kpt.TABLE_PARKER16, kpt.PRECISION_F64)
    with pytest.raises(kpt.KptError, match="mixed-precision"):
        batch.add_run(parts, lo64, lo64, parker, 1, 0)
    lo = ctx.field(f, kpt.TABLE_PARKER16, kpt.PRECISION_MIXED)
    batch.add_run(parts, lo, lo, parker, 1, 0)
    lof = ctx.field(f, kpt.TABLE_FOCUSED21, kpt.PRECISION_MIXED)
    parts2 = ctx.particles(8)
    with pytest.raises(kpt.KptError, match="transport model"):
        batch.add_run(parts2, lof, lof, focused, 1, 0)
    for h in (batch, parts, parts2, lo64, lo, lof):
        h.close()
