"""The CLI drop-in (kokkos_particle_transport_app) against the reference CLI.

tests/golden/cli/ holds a complete run of the reference's own CLI (two frames,
splitting near capacity, every output written) and a restart from its frame-2
snapshot; the same flags on the same fields must give the same files:
counts, ids, statuses, split levels and histogram weights exactly; positions,
momenta and pitch cosines within the FP64 parity bar; summary averages within
1e-12 (tree vs serial sums); timing columns are not compared.
"""
from __future__ import annotations

import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

pytestmark = pytest.mark.gpu

APP = os.path.join(ROOT, "kokkos-particletransport_gb300", "bin", "kokkos_particle_transport_app")
CLI = os.path.join(GOLDEN, "cli")
PHYSICS_COLUMNS_EXACT = ("frame", "stored", "active", "inactive", "max_split_level", "injected",
                         "split", "skipped_split_capacity", "weight_sum", "p_min", "p_max",
                         "dt_min", "dt_max", "time")
PHYSICS_COLUMNS_CLOSE = ("p_avg", "dt_avg")


@pytest.fixture(scope="module")
def field_dir(tmp_path_factory, fields_mod):
    out = tmp_path_factory.mktemp("fields")
    data = np.load(os.path.join(CLI, "fields.npz"))
    k = 0
    while f"frame{k}_b" in data.files:
        f = fields_mod.CompactField(data[f"frame{k}_x_edges"], data[f"frame{k}_y_edges"],
                                    data[f"frame{k}_b"], data[f"frame{k}_v"])
        fields_mod.write_compact_field(fields_mod.field_file_path(str(out), k), f)
        k += 1
    return str(out)


def _argv():
    return open(os.path.join(CLI, "argv.txt")).read().split()


def _run(args):
    proc = subprocess.run([APP] + args, capture_output=True, text=True, timeout=300)
    assert proc.returncode == 0, proc.stderr
    return proc


def _compare_summary(got_path, want_path, formats):
    got = formats.read_summary_csv(got_path)
    want = formats.read_summary_csv(want_path)
    assert len(got) == len(want)
    for g, w in zip(got, want):
        for key in PHYSICS_COLUMNS_EXACT:
            if key in ("weight_sum", "p_min", "p_max", "dt_min", "dt_max", "time"):
                assert float(g[key]) == pytest.approx(float(w[key]), rel=1e-10, abs=0), key
            else:
                assert g[key] == w[key], key
        for key in PHYSICS_COLUMNS_CLOSE:
            assert float(g[key]) == pytest.approx(float(w[key]), rel=1e-10), key


def _compare_snapshot(got_path, want_path, formats):
    got = formats.read_snapshot(got_path)
    want = formats.read_snapshot(want_path)
    assert (got.count, got.capacity, got.charge, got.split_ratio) == \
        (want.count, want.capacity, want.charge, want.split_ratio)
    g, w = got.records, want.records
    for key in ("id", "status", "split_level", "sort_key"):
        assert np.array_equal(g[key], w[key]), key
    assert np.array_equal(g["weight"], w["weight"])
    assert np.array_equal(g["initial_kinetic_energy"], w["initial_kinetic_energy"])
    for key, scale in (("position", np.array([2.0, 4.0])), ("p", None), ("mu", 1.0)):
        diff = np.abs(g[key] - w[key])
        if key == "position":
            diff = np.minimum(diff, scale - diff) / scale
        elif key == "p":
            diff = diff / np.abs(w[key])
        assert diff.max() <= 1e-10, (key, diff.max())


def _compare_histogram(got_path, want_path, formats):
    got = formats.read_histogram_csv(got_path)
    want = formats.read_histogram_csv(want_path)
    assert np.array_equal(got["bin"], want["bin"])
    assert np.array_equal(got["weight"], want["weight"])
    # edges: the CLI writes the contracted (FMA) form of the reference's
    # optimised build; the golden run was built unfused.  The two exponent
    # arguments differ by at most one rounding, i.e. ~1e-15 relative after exp.
    for key in ("p_left", "p_right"):
        assert np.all(np.abs(got[key] - want[key]) <= 1e-14 * want[key]), key


@pytest.mark.parametrize("prefetch", ["on", "off"])
def test_cli_run_and_restart_match_reference(tmp_path, field_dir, fields_mod, prefetch):
    import importlib
    formats = importlib.import_module("kokkos-particletransport_gb300.formats")
    run_dir = tmp_path / "run"
    _run(_argv() + ["--field-dir", field_dir, "--output-dir", str(run_dir), "--frames", "2",
                    "--frame-prefetch", prefetch])
    want_dir = os.path.join(CLI, "run")
    names = sorted(os.listdir(want_dir))
    assert sorted(os.listdir(run_dir)) == names
    _compare_summary(run_dir / "summary.csv", os.path.join(want_dir, "summary.csv"), formats)
    for name in names:
        if name.startswith("particles_"):
            _compare_snapshot(run_dir / name, os.path.join(want_dir, name), formats)
        elif name.startswith("momentum_histogram_"):
            _compare_histogram(run_dir / name, os.path.join(want_dir, name), formats)
    # restart from the frame-2 snapshot, appending to a copy of the reference's run
    restart_dir = tmp_path / "restart"
    restart_dir.mkdir()
    shutil.copy(os.path.join(CLI, "restart", "particles_00002.bin"), restart_dir)
    _run(_argv() + ["--field-dir", field_dir, "--output-dir", str(restart_dir),
                    "--restart-particle-snapshot", str(restart_dir / "particles_00002.bin"),
                    "--frames", "1"])
    want_restart = os.path.join(CLI, "restart")
    _compare_summary(restart_dir / "summary.csv", os.path.join(want_restart, "summary.csv"),
                     formats)
    _compare_snapshot(restart_dir / "particles_00003.bin",
                      os.path.join(want_restart, "particles_00003.bin"), formats)
    _compare_histogram(restart_dir / "momentum_histogram_00003.csv",
                       os.path.join(want_restart, "momentum_histogram_00003.csv"), formats)
    log = open(restart_dir / "run.log").read()
    assert "Restarted from particle snapshot" in log and "effective_seed=" in log


def test_cli_refuses_to_overwrite_and_reports_errors(tmp_path, field_dir):
    out = tmp_path / "out"
    _run(["--profile", "smoke", "--field-dir", field_dir, "--output-dir", str(out),
          "--particles-per-frame", "64", "--capacity", "256"])
    again = subprocess.run([APP, "--profile", "smoke", "--field-dir", field_dir,
                            "--output-dir", str(out)], capture_output=True, text=True)
    assert again.returncode == 1 and again.stderr.startswith("Error: Output directory already")
    missing = subprocess.run([APP, "--profile", "smoke", "--field-dir", str(tmp_path / "none"),
                              "--output-dir", str(tmp_path / "o2")], capture_output=True,
                             text=True)
    assert missing.returncode == 1 and "Error:" in missing.stderr
