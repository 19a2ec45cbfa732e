"""The 256x512 configuration (the reference's own CPU-runnable case).

* Harness mode: 25,600 particles injected in |y| < 0.2 at t0 = 0, p = p0,
  kappa_perp/kappa_par = 0.05, dt fixed at 1e-3 (dt_min_rel = dt_max_rel =
  1e-2), one interval = exactly 100 substeps per particle, FP64 push against
  the oracle at 1e-10; the 64-bin spectrum is the pairwise sum of the 128
  reference bins, bit for bit.
* The strict CLI run (`--profile smoke --frames 1 --particles-per-frame 1600
  --rank-scale 16 --capacity 65536 --overwrite-output`) against the
  reference CLI's own summary, 128-bin histogram and first 2048 snapshot
  records (tests/golden/c1/, made by tests/golden/make_golden.py).
"""
from __future__ import annotations

import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT
from test_gpu_cli import APP, _compare_histogram, _compare_summary

pytestmark = pytest.mark.gpu

C1 = os.path.join(GOLDEN, "c1")


def test_c1_harness_fixed_dt_hundred_steps(ctx, kpt, oracle, binding, fields_mod):
    field = fields_mod.harris_field(256, 512)
    params = binding.default_params(kperp_over_kpara=0.05, dt_min_rel=1e-2, dt_max_rel=1e-2)
    n = 25600
    grid = oracle.grid(field.x_edges, field.y_edges)
    start = binding.empty_particles(n)
    count = oracle.inject(grid, params, 0.0, 0, 114514, n, 0, n, start, band=(-0.2, 0.2))
    assert count == n
    start["t"][:count] = 0.0
    ref = {k: v.copy() for k, v in start.items()}
    table = oracle.table(field)
    steps = oracle.push(grid, table, table, params, 0.0, 0, 114514, count, ref)
    oracle.free_grid(grid)
    assert np.all(steps == 100)
    settings = kpt.settings_from_dict(params)
    lower = ctx.field(field)
    parts = ctx.particles(n)
    parts.upload(start, count)
    stats = ctx.push_interval(parts, lower, lower, settings, 0, 114514)
    assert stats.particle_steps == 100 * n and stats.max_steps == 100
    got = parts.download()
    for name in ("x", "y"):
        width = 2.0 if name == "x" else 4.0
        diff = np.abs(got[name] - ref[name][:count])
        assert (np.minimum(diff, width - diff) / width).max() <= 1e-10, name
    assert (np.abs(got["p"] - ref["p"][:count]) / ref["p"][:count]).max() <= 1e-10
    assert np.array_equal(got["status"], ref["status"][:count])
    # 64 log bins = pairwise sums of the reference's 128, exactly
    h128 = ctx.histogram(parts, params["pmin"], params["pmax"], 128)
    h64 = ctx.histogram(parts, params["pmin"], params["pmax"], 64)
    assert np.array_equal(h64, h128.reshape(64, 2).sum(axis=1))
    ref128 = oracle.histogram(params["pmin"], params["pmax"], 128, count, ref)
    assert np.array_equal(h128, ref128)
    for h in (parts, lower):
        h.close()


def test_c1_strict_cli_matches_reference(tmp_path, fields_mod):
    import importlib
    formats = importlib.import_module("kokkos-particletransport_gb300.formats")
    field = fields_mod.harris_field(256, 512)
    field_dir = tmp_path / "fields"
    field_dir.mkdir()
    for k in range(2):
        fields_mod.write_compact_field(fields_mod.field_file_path(str(field_dir), k), field)
    out = tmp_path / "run"
    argv = open(os.path.join(C1, "argv.txt")).read().split()
    proc = subprocess.run([APP] + argv + ["--field-dir", str(field_dir), "--output-dir",
                                          str(out)], capture_output=True, text=True, timeout=300)
    assert proc.returncode == 0, proc.stderr
    _compare_summary(out / "summary.csv", os.path.join(C1, "summary.csv"), formats)
    _compare_histogram(out / "momentum_histogram_00001.csv",
                       os.path.join(C1, "momentum_histogram_00001.csv"), formats)
    snap = formats.read_snapshot(str(out / "particles_00001.bin"))
    want = np.load(os.path.join(C1, "snapshot_head.npz"))
    assert snap.count == int(want["count"]) == 25600
    assert snap.capacity == int(want["capacity"])
    got = snap.records[:2048]
    for key in ("id", "status", "split_level", "sort_key", "weight", "initial_kinetic_energy"):
        assert np.array_equal(got[key], want[key]), key
    pos = np.abs(got["position"] - want["position"])
    pos = np.minimum(pos, np.array([2.0, 4.0]) - pos) / np.array([2.0, 4.0])
    assert pos.max() <= 1e-10
    assert (np.abs(got["p"] - want["p"]) / want["p"]).max() <= 1e-10
