"""Cell records of the mixed pushes.

A mixed push may sample per-cell records of its table pair (each
component's eight corner values of both frames in one 32-byte sector, read
by four cooperating lanes a 128-byte line at a time) instead of the
point-major tables.  The record sampler performs the point-major sampler's
operations in the same order, so every particle must end bit for bit where
the point-table push leaves it: both transports, uniform and stretched
axes, with and without time interpolation, partial warps (lanes without a
particle help sample), the plain closure and the learned closure on both
engines, and across a change of the table pair (the records are rebuilt).
"""
from __future__ import annotations

import numpy as np
import pytest

from test_gpu_surrogate import trained64  # noqa: F401  (module fixture)

pytestmark = pytest.mark.gpu


def _fields(fields_mod, nx, ny, stretched, seeds):
    ye = fields_mod.stretched_edges(ny, -2.0, 2.0) if stretched else None
    return [fields_mod.harris_field(nx, ny, y_edges=ye, island_amplitude=0.1, noise=0.02,
                                    seed=s) for s in seeds]


def _push_both_ways(ctx, kpt, tables, settings, start, n, frames, seed, sort=True):
    """The same population pushed over consecutive table pairs with the
    records off, then on; returns both end states and particle-step counts."""
    out = []
    parts = ctx.particles(n)
    try:
        for mode in (kpt.RECORDS_OFF, kpt.RECORDS_ON):
            ctx.set_cell_records(mode)
            parts.upload(start, n)
            steps = 0
            for k, frame in enumerate(frames):
                lower, upper = tables[k], tables[k + 1]
                if sort:
                    ctx.sort(parts, lower, 8, 8)
                stats = ctx.push_interval(parts, lower, upper, settings, frame, seed)
                steps += stats.particle_steps
            out.append((parts.download(n), steps))
    finally:
        ctx.set_cell_records(kpt.RECORDS_AUTO)
        parts.close()
    return out


def _assert_same(results):
    (a, steps_a), (b, steps_b) = results
    assert steps_a > 0
    assert steps_a == steps_b
    for name in a:
        assert np.array_equal(a[name], b[name]), name


@pytest.mark.parametrize("focused", [False, True])
@pytest.mark.parametrize("stretched", [False, True])
@pytest.mark.parametrize("time_interpolation", [1, 0])
def test_records_equal_point_tables(ctx, kpt, binding, fields_mod, focused, stretched,
                                    time_interpolation):
    params = binding.default_params(kperp_over_kpara=0.05, focused=int(focused),
                                    time_interpolation=time_interpolation)
    settings = kpt.settings_from_dict(params)
    kind = kpt.TABLE_FOCUSED21 if focused else kpt.TABLE_PARKER16
    fields = _fields(fields_mod, 48, 96, stretched, (31, 32, 33))
    tables = [ctx.field(f, kind, kpt.PRECISION_MIXED) for f in fields]
    n = 2999  # not a multiple of the warp: partial warps at the end of the cursor
    parts = ctx.particles(n)
    ctx.inject(parts, tables[0], settings, n, 4, 17)
    start = parts.download(n)
    parts.close()
    try:
        # two intervals over three frames: the second pair rebuilds the records
        _assert_same(_push_both_ways(ctx, kpt, tables, settings, start, n, (4, 5), 17))
    finally:
        for t in tables:
            t.close()


@pytest.mark.parametrize("engine", ["tcgen05", "mma.sync"])
def test_records_equal_point_tables_learned_closure(ctx, kpt, fields_mod, trained64, engine):
    _, settings, surrogate = trained64
    default_engine = surrogate.engine
    surrogate.engine = kpt.ENGINE_TCGEN05 if engine == "tcgen05" else kpt.ENGINE_MMA_SYNC
    fields = _fields(fields_mod, 64, 128, True, (5, 6))
    tables = [ctx.field(f, kpt.TABLE_FOCUSED21, kpt.PRECISION_MIXED) for f in fields]
    ctx.set_surrogate(surrogate)
    n = 5000
    parts = ctx.particles(n)
    ctx.inject(parts, tables[0], settings, n, 7, 99)
    start = parts.download(n)
    parts.close()
    try:
        _assert_same(_push_both_ways(ctx, kpt, tables, settings, start, n, (7,), 99))
        # unsorted work order: the lanes of a group sample unrelated cells
        _assert_same(_push_both_ways(ctx, kpt, tables, settings, start, n, (7,), 99,
                                     sort=False))
    finally:
        surrogate.engine = default_engine
        ctx.set_surrogate(None)
        for t in tables:
            t.close()


@pytest.mark.parametrize("focused", [False, True])
@pytest.mark.parametrize("shape", [(128, 1), (256, 2)])
def test_batched_records_equal_point_tables(ctx, kpt, fields_mod, binding, oracle, focused,
                                            shape):
    """Batched runs (lanes of one warp in different runs, each sampling its
    run's records), one run without time interpolation among runs with it
    (a warp that mixes them samples the point tables for that substep)."""
    from test_gpu_batch import _runs, _tables
    runs = _runs(kpt, fields_mod, binding, oracle, focused)
    params = binding.default_params(kperp_over_kpara=0.05, focused=int(focused),
                                    time_interpolation=0)
    runs[1]["settings"] = kpt.settings_from_dict(params)
    results = []
    try:
        for mode in (kpt.RECORDS_OFF, kpt.RECORDS_ON):
            ctx.set_cell_records(mode)
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
            batch.run(2, use_graph=True)
            results.append([h[0].download() for h in handles])
            batch.close()
            for h in handles:
                for x in h:
                    x.close()
    finally:
        ctx.set_cell_records(kpt.RECORDS_AUTO)
    for a, b in zip(*results):
        for name in a:
            assert np.array_equal(a[name], b[name]), name


def test_records_reused_on_another_stream(ctx, kpt, binding, fields_mod):
    """Records built on one stream and reused by a push on another (the
    caller switched the context's stream): the second push is ordered after
    the build and ends where the point-table push does."""
    import torch
    params = binding.default_params(kperp_over_kpara=0.05, focused=1)
    settings = kpt.settings_from_dict(params)
    fields = _fields(fields_mod, 48, 96, True, (41, 42))
    tables = [ctx.field(f, kpt.TABLE_FOCUSED21, kpt.PRECISION_MIXED) for f in fields]
    n = 3000
    parts = ctx.particles(n)
    ctx.inject(parts, tables[0], settings, n, 4, 23)
    start = parts.download(n)
    first, second = torch.cuda.Stream(), torch.cuda.Stream()
    results = []
    try:
        for mode in (kpt.RECORDS_OFF, kpt.RECORDS_ON):
            ctx.set_cell_records(mode)
            for stream in (first, second):
                ctx.set_stream(stream.cuda_stream)
                parts.upload(start, n)
                ctx.push_interval(parts, tables[0], tables[1], settings, 4, 23)
                results.append(parts.download(n))
    finally:
        ctx.set_stream(0)  # back to the context's own stream
        ctx.set_cell_records(kpt.RECORDS_AUTO)
        parts.close()
        for t in tables:
            t.close()
    for other in results[1:]:
        for name in results[0]:
            assert np.array_equal(results[0][name], other[name]), name


def test_records_mode_is_checked(ctx, kpt):
    with pytest.raises(kpt.KptError):
        ctx.set_cell_records(7)
