"""GPU parity: the CUDA library (through the C ABI) against the oracle and the
reference's golden vectors.

Bars: integer/index work (tables in FP64, injection, split, histogram bins,
counts) bit-exact; FP64 trajectories within 1e-10 relative (positions
relative to the periodic width); mixed precision within the tolerances stated
per test.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden_field, golden_params, golden_particles, load_golden
from parity import F64_REL, trajectory_errors

pytestmark = pytest.mark.gpu

PUSH_CASES = ["parker_uniform", "parker_fixed_dt", "parker_stretched", "focused_uniform",
              "focused_stretched"]


def _kind(kpt, focused):
    return kpt.TABLE_FOCUSED21 if focused else kpt.TABLE_PARKER16


@pytest.mark.parametrize("name", ["tables_uniform.npz", "tables_stretched.npz"])
def test_table_f64_bit_exact(ctx, kpt, oracle, name):
    data = load_golden(name)
    field = golden_field(data, "field")
    for focused, key in ((False, "parker"), (True, "focused")):
        got = ctx.field(field, _kind(kpt, focused), kpt.PRECISION_F64).table()
        want = oracle.table(field, focused=focused)
        if name == "tables_uniform.npz":
            assert np.array_equal(want, data[key])
        assert np.array_equal(got, want), key


def test_table_mixed_is_rounded_f64(ctx, kpt, oracle):
    data = load_golden("tables_uniform.npz")
    field = golden_field(data, "field")
    for focused in (False, True):
        got = ctx.field(field, _kind(kpt, focused), kpt.PRECISION_MIXED).table()
        want = oracle.table(field, focused=focused).astype(np.float32).astype(np.float64)
        assert np.array_equal(got, want)


def test_inject_bit_exact(ctx, kpt):
    data = load_golden("inject.npz")
    params = golden_params(data)
    settings = kpt.settings_from_dict(params)
    field = ctx.field(golden_field(data, "field"))
    cap, frame, seed = int(data["capacity"]), int(data["frame"]), int(data["seed"])
    for key, count0, band in (("full", 0, (0.0, 0.0)), ("band", 0, (-0.2, 0.2)),
                              ("clamp", 2500, (0.0, 0.0))):
        parts = ctx.particles(cap)
        if count0:
            init = golden_particles(data, key)
            start = {k: np.zeros_like(v) for k, v in init.items()}
            start["status"][:] = 2
            start["status"][:count0] = 0
            parts.upload(start, count0)
        n = ctx.inject(parts, field, settings, 1000, frame, seed, band)
        assert parts.count == int(data[f"n_{key}"])
        assert n == int(data[f"n_{key}"]) - count0
        got = parts.download()
        want = golden_particles(data, key)
        for name in want:
            assert np.array_equal(got[name], want[name][: parts.count]), (key, name)


def _push_case(ctx, kpt, oracle, case, precision, max_steps=None):
    data = load_golden(f"push_{case}.npz")
    params = golden_params(data)
    if max_steps is not None:
        params["max_steps"] = max_steps
    focused = bool(params["focused"])
    lower_f = golden_field(data, "lower")
    upper_f = golden_field(data, "upper")
    count = int(data["count"])
    frame, seed = int(data["frame"]), int(data["seed"])
    start = golden_particles(data, "start")
    # Oracle on the same per-axis grid maps as the library (uniform x stays
    # analytic); for uniform cases this equals the golden end state.
    grid = oracle.grid(lower_f.x_edges, lower_f.y_edges)
    want = {k: v.copy() for k, v in start.items()}
    steps = oracle.push(grid, oracle.table(lower_f, focused), oracle.table(upper_f, focused),
                        params, frame * params["mhd_dt"], frame, seed, count, want)
    if "stretched" not in case and max_steps is None:
        golden_end = golden_particles(data, "end")
        for name in want:
            assert np.array_equal(want[name], golden_end[name])
    settings = kpt.settings_from_dict(params)
    kind = _kind(kpt, focused)
    lower = ctx.field(lower_f, kind, precision)
    upper = ctx.field(upper_f, kind, precision)
    parts = ctx.particles(count)
    parts.upload(start, count)
    stats = ctx.push_interval(parts, lower, upper, settings, frame, seed)
    got = parts.download()
    widths = (grid.upper[0] - grid.lower[0], grid.upper[1] - grid.lower[1])
    oracle.free_grid(grid)
    return got, want, steps, stats, widths, focused


# Focused transport runs ~7000 substeps per interval and its pitch-angle
# dynamics amplify any last-bit difference.  The FP64 push therefore rounds
# exactly as the oracle does: no FMA contraction (its own translation unit,
# -fmad=false, as the oracle and the reference build use -ffp-contract=off)
# and the same pow (kpt_pow.h, compared bit for bit below).  The 1e-10 bar
# holds over the first 1000 substeps and over the whole interval.
FOCUSED_PARITY_STEPS = 1000
FOCUSED_INTERVAL_REL = F64_REL


def test_pow_on_gpu_is_the_oracles_bit_for_bit(ctx, oracle):
    rng = np.random.default_rng(21)
    n = 200_000
    x = np.concatenate([np.exp(rng.uniform(-8, 8, n)), rng.uniform(0, 1, n),
                        np.exp(rng.uniform(-700, 700, n)), 1 + rng.uniform(-1e-3, 1e-3, n),
                        -np.exp(rng.uniform(-3, 3, 1000)), [0.0, -0.0, np.inf, -np.inf, np.nan,
                                                            1e-310, 1.0, -1.0, 2.0]])
    y = np.concatenate([rng.uniform(-3, 3, n), np.full(n, 5.0 / 3.0 - 2.0),
                        rng.uniform(-1, 1, n), rng.uniform(-50, 50, n),
                        rng.integers(-5, 6, 1000).astype(float),
                        [0.5, 3.0, -0.5, 3.0, 2.0, 0.5, np.nan, np.inf, -1074.5]])
    got = ctx.pow(x, y)
    want = oracle.pow(x, y)
    same = (got.view(np.uint64) == want.view(np.uint64)) | (np.isnan(got) & np.isnan(want))
    assert same.all(), (x[~same][:5], y[~same][:5], got[~same][:5], want[~same][:5])


@pytest.mark.parametrize("case", PUSH_CASES)
def test_push_f64_matches_oracle(ctx, kpt, oracle, case):
    focused_case = case.startswith("focused")
    got, want, steps, stats, widths, focused = _push_case(
        ctx, kpt, oracle, case, kpt.PRECISION_F64,
        FOCUSED_PARITY_STEPS if focused_case else None)
    errs = trajectory_errors(got, want, widths[0], widths[1], focused)
    for name, err in errs.items():
        assert err <= F64_REL, (name, err)
    assert np.array_equal(got["status"], want["status"])
    assert np.array_equal(got["w"], want["w"]) and np.array_equal(got["level"], want["level"])
    assert stats.particle_steps == int(steps.sum())
    assert stats.max_steps == int(steps.max())
    assert stats.pushed == int(np.count_nonzero(golden_particles(
        load_golden(f"push_{case}.npz"), "start")["status"] == 0))


@pytest.mark.parametrize("case", ["focused_uniform", "focused_stretched"])
def test_push_f64_focused_whole_interval(ctx, kpt, oracle, case):
    got, want, steps, stats, widths, focused = _push_case(ctx, kpt, oracle, case,
                                                         kpt.PRECISION_F64)
    errs = trajectory_errors(got, want, widths[0], widths[1], focused)
    print(case, "whole interval", {k: float(v) for k, v in errs.items()},
          "substeps", int(steps.sum()))
    for name, err in errs.items():
        assert err <= FOCUSED_INTERVAL_REL, (name, err)
    assert np.array_equal(got["status"], want["status"])
    assert stats.particle_steps == int(steps.sum())


@pytest.mark.parametrize("case", [c for c in PUSH_CASES if c.startswith("parker")])
def test_push_mixed_parker_within_tolerance(ctx, kpt, oracle, case):
    """Mixed precision (FP32 table, interpolation, coefficients and noise;
    fixed-point position, FP64 time and momentum) against the FP64 oracle over
    a whole Parker interval.  Stated tolerance: positions 1e-6 of the domain
    width, momentum 1e-6 relative, time 1e-12 relative; every status equal
    and substep counts within 1 %."""
    got, want, steps, stats, widths, focused = _push_case(ctx, kpt, oracle, case,
                                                         kpt.PRECISION_MIXED)
    errs = trajectory_errors(got, want, widths[0], widths[1], focused)
    assert errs["x"] <= 1e-6 and errs["y"] <= 1e-6, errs
    assert errs["p"] <= 1e-6, errs
    assert errs["t"] <= 1e-12, errs
    assert np.array_equal(got["status"], want["status"])
    assert abs(stats.particle_steps - int(steps.sum())) <= 0.01 * steps.sum() + 2


@pytest.mark.parametrize("case", ["focused_uniform", "focused_stretched"])
def test_push_mixed_focused_short_run(ctx, kpt, oracle, case):
    """Focused mixed precision over the first 50 substeps (beyond that the
    pitch-angle dynamics decorrelate FP32 and FP64 trajectories and only the
    statistics are compared): positions 1e-6 of the width, p 1e-6, mu 1e-4."""
    got, want, steps, stats, widths, focused = _push_case(ctx, kpt, oracle, case,
                                                         kpt.PRECISION_MIXED, 50)
    errs = trajectory_errors(got, want, widths[0], widths[1], focused)
    assert errs["x"] <= 1e-6 and errs["y"] <= 1e-6, errs
    assert errs["p"] <= 1e-6, errs
    assert errs["mu"] <= 1e-4, errs
    assert np.array_equal(got["status"], want["status"])


def test_split_bit_exact(ctx, kpt):
    data = load_golden("split.npz")
    params = golden_params(data)
    settings = kpt.settings_from_dict(params)
    count = int(data["count"])
    for prefix, cap_key, n_key, s_key, k_key in (
            ("end", "capacity", "new_count", "split", "skipped"),
            ("small_end", "small_capacity", "small_new_count", "small_split", "small_skipped")):
        cap = int(data[cap_key])
        parts = ctx.particles(cap)
        start = {k: v[:cap] for k, v in golden_particles(data, "start").items()}
        parts.upload(start, count)
        split, skipped = ctx.split(parts, settings)
        assert (parts.count, split, skipped) == (int(data[n_key]), int(data[s_key]),
                                                 int(data[k_key]))
        got = parts.download(parts.count)
        want = golden_particles(data, prefix)
        for name in want:
            assert np.array_equal(got[name], want[name][: parts.count]), (prefix, name)


def _snapshot_particles(kpt):
    formats = pytest.importorskip("importlib").import_module(
        "kokkos-particletransport_gb300.formats")
    import os
    from conftest import GOLDEN
    snap = formats.read_snapshot(os.path.join(GOLDEN, "cli", "run", "particles_00002.bin"))
    return formats, snap


def test_histogram_matches_reference_csv(ctx, kpt, oracle):
    formats, snap = _snapshot_particles(kpt)
    import os
    from conftest import GOLDEN
    arrays = snap.to_arrays()
    parts = ctx.particles(snap.count)
    parts.upload(arrays, snap.count)
    bins = ctx.histogram(parts, 1e-2, 1e1, 128)
    csv = formats.read_histogram_csv(os.path.join(GOLDEN, "cli", "run",
                                                  "momentum_histogram_00002.csv"))
    assert np.array_equal(bins, csv["weight"])
    assert np.array_equal(bins, oracle.histogram(1e-2, 1e1, 128, snap.count, arrays))
    bins64 = ctx.histogram(parts, 1e-2, 1e1, 64)
    assert np.array_equal(bins64, bins.reshape(64, 2).sum(axis=1))


def test_histogram_edge_particles_rebinned_exactly(ctx, kpt, oracle, binding):
    """Momenta placed exactly on and one ulp either side of bin edges."""
    nbins, pmin, pmax = 64, 1e-2, 1e1
    edges = np.exp(np.log(pmin) + np.arange(1, nbins) * (np.log(pmax) - np.log(pmin)) / nbins)
    p = np.concatenate([edges, np.nextafter(edges, 0), np.nextafter(edges, 1), [pmin, pmax]])
    n = p.size
    arrays = binding.empty_particles(n)
    arrays["p"][:] = p
    arrays["w"][:] = 0.5 ** (np.arange(n) % 5)
    arrays["status"][:] = 0
    parts = ctx.particles(n)
    parts.upload(arrays, n)
    got = ctx.histogram(parts, pmin, pmax, nbins)
    assert np.array_equal(got, oracle.histogram(pmin, pmax, nbins, n, arrays))


def test_summary_matches_oracle(ctx, kpt, oracle):
    formats, snap = _snapshot_particles(kpt)
    arrays = snap.to_arrays()
    arrays["dt"][:] = np.linspace(1e-5, 1e-3, snap.count)
    arrays["status"][::7] = 2
    parts = ctx.particles(snap.count)
    parts.upload(arrays, snap.count)
    got = ctx.summarize(parts)
    want = oracle.summarize(snap.count, arrays)
    for key in ("stored", "active", "inactive", "max_split_level", "p_min", "p_max", "dt_min",
                "dt_max", "weight_sum"):
        assert got[key] == want[key], key
    for key in ("p_avg", "dt_avg"):
        assert got[key] == pytest.approx(want[key], rel=1e-13), key


def test_sample_matches_oracle(ctx, kpt, oracle):
    data = load_golden("push_parker_stretched.npz")
    lower_f = golden_field(data, "lower")
    upper_f = golden_field(data, "upper")
    rng = np.random.default_rng(3)
    n = 4000
    x = rng.uniform(-1.3, 1.3, n)
    y = rng.uniform(-2.5, 2.5, n)
    rt = rng.uniform(-0.2, 1.2, n)
    for focused in (False, True):
        kind = _kind(kpt, focused)
        lower = ctx.field(lower_f, kind, kpt.PRECISION_F64)
        upper = ctx.field(upper_f, kind, kpt.PRECISION_F64)
        got = ctx.sample(lower, upper, x, y, rt)
        grid = oracle.grid(lower_f.x_edges, lower_f.y_edges)
        lt, ut = oracle.table(lower_f, focused), oracle.table(upper_f, focused)
        want = np.stack([_oracle_sample(oracle, grid, lt, ut, 21 if focused else 16,
                                        x[i], y[i], rt[i]) for i in range(n)])
        oracle.free_grid(grid)
        scale = np.maximum(np.abs(want).max(axis=0), 1e-30)
        assert np.max(np.abs(got - want) / scale) < 1e-13


def _oracle_sample(oracle, grid, lt, ut, ncomp, x, y, rt):
    import ctypes
    lower, upper = grid.lower, grid.upper
    xw = oracle.wrap(x, lower[0], upper[0], upper[0] - lower[0])
    yw = oracle.wrap(y, lower[1], upper[1], upper[1] - lower[1])
    out = np.zeros(ncomp)
    oracle.lib.kpt_oracle_sample(ctypes.byref(grid), lt.ctypes.data_as(ctypes.c_void_p),
                                 ut.ctypes.data_as(ctypes.c_void_p), ncomp, xw, yw, rt, 1,
                                 out.ctypes.data_as(ctypes.c_void_p))
    return out


def test_step_guard_and_empty(ctx, kpt, oracle):
    data = load_golden("push_parker_uniform.npz")
    params = golden_params(data)
    params["max_steps"] = 3
    lower_f = golden_field(data, "lower")
    upper_f = golden_field(data, "upper")
    count = int(data["count"])
    frame, seed = int(data["frame"]), int(data["seed"])
    start = golden_particles(data, "start")
    grid = oracle.grid(lower_f.x_edges, lower_f.y_edges)
    want = {k: v.copy() for k, v in start.items()}
    oracle.push(grid, oracle.table(lower_f), oracle.table(upper_f), params,
                frame * params["mhd_dt"], frame, seed, count, want)
    oracle.free_grid(grid)
    settings = kpt.settings_from_dict(params)
    lower, upper = ctx.field(lower_f), ctx.field(upper_f)
    parts = ctx.particles(count)
    parts.upload(start, count)
    stats = ctx.push_interval(parts, lower, upper, settings, frame, seed)
    got = parts.download()
    assert np.array_equal(got["status"], want["status"])
    assert stats.failed == int(np.count_nonzero((want["status"] == 2) &
                                                (start["status"] == 0)))
    assert stats.failed > 0
    empty = ctx.particles(16)
    stats = ctx.push_interval(empty, lower, upper, settings, frame, seed)
    assert stats.particle_steps == 0 and stats.pushed == 0


def test_zero_field_marks_failed(ctx, kpt, fields_mod, binding):
    """|B| = 0 in the sampled cells sets status 2 (src/main.cpp:1167-1171)."""
    f = fields_mod.harris_field(16, 16, guide=0.0, perturbation=0.0)
    f.b[:] = 0.0
    params = binding.default_params()
    settings = kpt.settings_from_dict(params)
    lower = ctx.field(f)
    parts = ctx.particles(64)
    ctx.inject(parts, lower, settings, 64, 0, 5)
    stats = ctx.push_interval(parts, lower, lower, settings, 0, 5)
    got = parts.download()
    assert np.all(got["status"] == 2)
    assert stats.failed == 64 and stats.particle_steps == 64


def test_bad_arguments_raise(ctx, kpt, fields_mod):
    f = fields_mod.harris_field(8, 8)
    with pytest.raises(kpt.KptError):
        ctx.particles(0)
    bad = fields_mod.CompactField(f.x_edges[::-1].copy(), f.y_edges, f.b, f.v)
    with pytest.raises(kpt.KptError):
        ctx.field(bad)
    nan = fields_mod.CompactField(f.x_edges, f.y_edges, f.b.copy(), f.v)
    nan.b[0, 0, 0] = np.nan
    with pytest.raises(kpt.KptError):
        ctx.field(nan)
    lower = ctx.field(f)
    focused = ctx.field(f, kpt.TABLE_FOCUSED21)
    parts = ctx.particles(8)
    with pytest.raises(kpt.KptError):
        ctx.push_interval(parts, lower, focused, kpt.default_settings(), 0, 1)
    with pytest.raises(kpt.KptError):
        ctx.push_interval(parts, lower, lower, kpt.default_settings(charge=0.0), 0, 1)


@pytest.mark.parametrize("case", ["focused_uniform", "focused_stretched"])
def test_push_f64_qlt_closure_matches_oracle(ctx, kpt, oracle, case):
    """Focused push with the slab-QLT closure (LegencyModel D_mumu, dD_mumu/dmu;
    the oracle's closure is bit-identical to the reference's functions)."""
    data = load_golden(f"push_{case}.npz")
    params = golden_params(data)
    params.update(closure=1, max_steps=FOCUSED_PARITY_STEPS)
    lower_f = golden_field(data, "lower")
    upper_f = golden_field(data, "upper")
    count = int(data["count"])
    frame, seed = int(data["frame"]), int(data["seed"])
    start = golden_particles(data, "start")
    grid = oracle.grid(lower_f.x_edges, lower_f.y_edges)
    want = {k: v.copy() for k, v in start.items()}
    steps = oracle.push(grid, oracle.table(lower_f, True), oracle.table(upper_f, True), params,
                        frame * params["mhd_dt"], frame, seed, count, want)
    widths = (grid.upper[0] - grid.lower[0], grid.upper[1] - grid.lower[1])
    oracle.free_grid(grid)
    settings = kpt.settings_from_dict(params)
    lower = ctx.field(lower_f, kpt.TABLE_FOCUSED21, kpt.PRECISION_F64)
    upper = ctx.field(upper_f, kpt.TABLE_FOCUSED21, kpt.PRECISION_F64)
    parts = ctx.particles(count)
    parts.upload(start, count)
    stats = ctx.push_interval(parts, lower, upper, settings, frame, seed)
    got = parts.download()
    errs = trajectory_errors(got, want, widths[0], widths[1], True)
    for name, err in errs.items():
        assert err <= F64_REL, (name, err)
    assert np.array_equal(got["status"], want["status"])
    assert stats.particle_steps == int(steps.sum())


def test_snapshot_records_packed_on_gpu(ctx, kpt):
    """v4 records of write_reconnection_particle_snapshot (src/main.cpp:2155-2201)
    packed by the GPU: byte-identical to records built on the host from the
    downloaded arrays."""
    import importlib
    formats = importlib.import_module("kokkos-particletransport_gb300.formats")
    data = load_golden("push_parker_uniform.npz")
    n = int(data["count"])
    parts = ctx.particles(n + 5)
    parts.upload(golden_particles(data, "end"), n)
    e0 = float(np.sqrt(1.0 + 0.1 ** 2) - 1.0)
    got = parts.pack_records(e0)
    host = parts.download()
    want = np.zeros(n, dtype=formats.RECORD_DTYPE)
    want["id"] = np.arange(n)
    want["status"] = host["status"]
    want["split_level"] = host["level"]
    xy = np.stack([host["x"], host["y"]], axis=1)
    for key in ("position", "previous_position", "previous_step_position"):
        want[key] = xy
    want["p"], want["mu"], want["weight"] = host["p"], host["mu"], host["w"]
    want["initial_kinetic_energy"] = e0
    assert got.tobytes() == want.tobytes()
    parts.close()


@pytest.mark.parametrize("case", ["parker_uniform", "focused_uniform"])
def test_push_f64_contracted_stays_close_to_strict(ctx, kpt, oracle, case):
    """The contracted FP64 arithmetic (FMA fusion, CUDA's pow) is the faster
    FP64 push; it leaves the oracle's trajectories by last-bit differences
    only: within the 1e-10 bar over a Parker interval and over the first
    1000 focused substeps (the focused pitch-angle dynamics amplify them
    later in the interval)."""
    focused_case = case.startswith("focused")
    ctx.set_fp64_arithmetic(kpt.FP64_CONTRACTED)
    try:
        got, want, steps, stats, widths, focused = _push_case(
            ctx, kpt, oracle, case, kpt.PRECISION_F64,
            FOCUSED_PARITY_STEPS if focused_case else None)
    finally:
        ctx.set_fp64_arithmetic(kpt.FP64_STRICT)
    errs = trajectory_errors(got, want, widths[0], widths[1], focused)
    print(case, "contracted", errs)
    for name, err in errs.items():
        assert err <= F64_REL, (name, err)
    assert np.array_equal(got["status"], want["status"])
