"""The oracle restatement against golden vectors made by the reference itself.

Every fixture under tests/golden/ was produced by the reference's own driver
code (tests/golden/make_golden.py); the oracle must reproduce it bit for bit.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden_field, golden_params, golden_particles, load_golden

PUSH_CASES = ["parker_uniform", "parker_fixed_dt", "parker_stretched", "focused_uniform",
              "focused_stretched"]


@pytest.mark.parametrize("name", ["tables_uniform.npz", "tables_stretched.npz"])
def test_tables_bit_exact(oracle, name):
    data = load_golden(name)
    field = golden_field(data, "field")
    stretched = "stretched" in name
    for focused, key in ((False, "parker"), (True, "focused")):
        got = oracle.table(field, focused=focused, force_stored=stretched)
        assert got.shape == data[key].shape
        assert np.array_equal(got, data[key]), key


def test_inject_bit_exact(oracle, binding):
    data = load_golden("inject.npz")
    params = golden_params(data)
    field = golden_field(data, "field")
    grid = oracle.grid(field.x_edges, field.y_edges)
    cap, frame, seed = int(data["capacity"]), int(data["frame"]), int(data["seed"])
    start = frame * params["mhd_dt"]
    for key, count0, band in (("full", 0, (0.0, 0.0)), ("band", 0, (-0.2, 0.2)),
                              ("clamp", 2500, (0.0, 0.0))):
        parts = binding.empty_particles(cap)
        parts["status"][:count0] = 0
        n = oracle.inject(grid, params, start, frame, seed, cap, count0, 1000, parts, band=band)
        assert n == int(data[f"n_{key}"])
        want = golden_particles(data, key)
        for name in want:
            assert np.array_equal(parts[name], want[name]), (key, name)
    oracle.free_grid(grid)


@pytest.mark.parametrize("case", PUSH_CASES)
def test_push_bit_exact(oracle, case):
    data = load_golden(f"push_{case}.npz")
    params = golden_params(data)
    lower = golden_field(data, "lower")
    upper = golden_field(data, "upper")
    stretched = "stretched" in case
    focused = bool(params["focused"])
    grid = oracle.grid(lower.x_edges, lower.y_edges, force_stored=stretched)
    count = int(data["count"])
    frame, seed = int(data["frame"]), int(data["seed"])
    parts = golden_particles(data, "start")
    steps = oracle.push(grid, oracle.table(lower, focused, stretched),
                        oracle.table(upper, focused, stretched), params,
                        frame * params["mhd_dt"], frame, seed, count, parts)
    want = golden_particles(data, "end")
    for name in want:
        assert np.array_equal(parts[name], want[name]), name
    assert steps.sum() > 0
    assert steps[-1] == 0  # the inactive particle is not pushed
    oracle.free_grid(grid)


def test_split_bit_exact(oracle):
    data = load_golden("split.npz")
    params = golden_params(data)
    count = int(data["count"])
    for prefix, cap_key, n_key, s_key, k_key in (
            ("end", "capacity", "new_count", "split", "skipped"),
            ("small_end", "small_capacity", "small_new_count", "small_split", "small_skipped")):
        cap = int(data[cap_key])
        parts = {k: v[:cap].copy() for k, v in golden_particles(data, "start").items()}
        n, s, k = oracle.split(params, cap, count, parts)
        assert (n, s, k) == (int(data[n_key]), int(data[s_key]), int(data[k_key]))
        want = golden_particles(data, prefix)
        for name in want:
            assert np.array_equal(parts[name][:cap], want[name][:cap]), (prefix, name)


def test_wrap_matches_reference_branches(oracle):
    lower, upper = -1.0, 1.0
    width = upper - lower
    for value, expect in ((0.5, 0.5), (1.0, -1.0), (-1.0, -1.0), (1.5, -0.5), (-1.5, 0.5),
                          (7.25, -0.75), (-9.0, -1.0)):
        assert oracle.wrap(value, lower, upper, width) == pytest.approx(expect, abs=1e-15)


def test_qlt_closure_bit_exact(oracle):
    """Slab-QLT D_mumu and dD_mumu/dmu: the reference's LegencyModel functions."""
    data = load_golden("qlt_closure.npz")
    d, dd = oracle.qlt(data["mu"], data["omega"], data["speed"], data["sigma2"], data["lc"],
                       data["gk"], data["h0"])
    assert np.array_equal(d, data["dmumu"])
    assert np.array_equal(dd, data["dmumu_dmu"])
    assert np.all(data["dmumu"] >= 0.0)
    assert data["dmumu"][np.abs(data["mu"]) == 1.0].max() == 0.0
