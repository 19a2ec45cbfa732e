"""The C++ drop-in headers (include/kpt/*.hpp) against the reference.

tests/cpp/solver_api_check.cpp (built by build() into
kokkos-particletransport_gb300/bin/kpt_solver_api_check) drives
kpt::ParkerSolver, kpt::FocusSolver and kpt::ParticleSystem as a user of the
reference's header library drives ParkerSolver / FocusSolver /
ParticleSystem (constructors from particles, grid, B, V and coefficients;
compute_adaptive_time_step, advance_stochastic(RandomManager),
advance_deterministic; the lifecycle calls).  Its results are compared with
the reference's golden vectors (tests/golden/lib_*.npz, made by the
reference's own templates) at the bars of tests/test_gpu_library.py: dt
within 1e-12 (focused 1e-10), states within 1e-10, integer fields exact;
lifecycle operations bit for bit.  The error paths keep the reference's
messages.
"""
from __future__ import annotations

import os
import struct
import subprocess

import numpy as np
import pytest

from conftest import ROOT, load_golden

pytestmark = pytest.mark.gpu

CHECK = os.path.join(ROOT, "kokkos-particletransport_gb300", "bin", "kpt_solver_api_check")
FIELDS = ("id", "x", "y", "prev_x", "prev_y", "prevstep_x", "prevstep_y", "p", "mu", "w", "e0",
          "status", "level", "key")
TYPES = {"d": np.float64, "i": np.int32, "u": np.uint64}


def _write(path, records):
    with open(path, "wb") as out:
        for name, values in records.items():
            arr = np.atleast_1d(np.asarray(values))
            if arr.dtype == np.int32:
                code = "i"
            elif arr.dtype == np.uint64:
                code = "u"
            else:
                code, arr = "d", arr.astype(np.float64)
            out.write(name.encode().ljust(32, b"\0"))
            out.write(code.encode() + b"\0" * 7)
            out.write(struct.pack("<Q", arr.size))
            out.write(np.ascontiguousarray(arr).tobytes())


def _read(path):
    out = {}
    with open(path, "rb") as stream:
        data = stream.read()
    pos = 0
    while pos < len(data):
        name = data[pos:pos + 32].rstrip(b"\0").decode()
        code = chr(data[pos + 32])
        (count,) = struct.unpack("<Q", data[pos + 40:pos + 48])
        dtype = TYPES[code]
        size = count * np.dtype(dtype).itemsize
        out[name] = np.frombuffer(data[pos + 48:pos + 48 + size], dtype=dtype).copy()
        pos += 48 + size
    return out


def _run(tmp_path, mode, records):
    assert os.path.exists(CHECK), "build() makes the C++ check program"
    src, dst = tmp_path / f"{mode}_in.bin", tmp_path / f"{mode}_out.bin"
    _write(src, records)
    proc = subprocess.run([CHECK, mode, str(src), str(dst)], capture_output=True, text=True,
                          timeout=300)
    assert proc.returncode == 0, proc.stderr
    return _read(dst)


def _inputs(data, keys):
    rec = {k: data[k] for k in keys}
    rec["periodic"] = np.asarray(data["periodic"], dtype=np.int32)
    for k in FIELDS:
        v = data[f"start_{k}"]
        rec[f"start_{k}"] = v.astype(np.uint64) if k == "id" else (
            v.astype(np.int32) if k in ("status", "level", "key") else v)
    return rec


def _text(codes):
    return "".join(chr(int(c)) for c in codes)


def _compare_state(got, want, prefix, data, rtol=1e-10):
    for key in ("status", "level", "key", "id", "w", "e0"):
        assert np.array_equal(got[f"{prefix}_{key}"], want[f"end_{key}"]), key
    wx = data["x_edges"][-1] - data["x_edges"][0]
    wy = data["y_edges"][-1] - data["y_edges"][0]
    for key, width in (("x", wx), ("prev_x", wx), ("prevstep_x", wx), ("y", wy), ("prev_y", wy),
                       ("prevstep_y", wy)):
        diff = np.abs(got[f"{prefix}_{key}"] - want[f"end_{key}"])
        diff = np.minimum(diff, np.abs(width - diff)) / width
        assert diff.max() <= rtol, (key, diff.max())
    for key in ("p", "mu"):
        scale = np.maximum(np.abs(want[f"end_{key}"]), 1e-12)
        assert (np.abs(got[f"{prefix}_{key}"] - want[f"end_{key}"]) / scale).max() <= rtol, key


@pytest.mark.parametrize("kind,case", [("parker", "readme_periodic"), ("parker", "ratio_open"),
                                       ("parker", "readme_deterministic"),
                                       ("focus", "readme_periodic"),
                                       ("focus", "ratio_open_mumax"), ("focus", "deterministic"),
                                       ("parker", "stored_ratio_open"),
                                       ("focus", "stored_ratio_open_mumax")])
def test_cxx_solver_steps_match_reference(tmp_path, kind, case):
    data = load_golden(f"lib_{kind}_{case}.npz")
    keys = ["x_edges", "y_edges", "count", "basis", "constant_ratio", "courant", "seed",
            "first_step", "steps", "stochastic"]
    if "x_faces" in data:  # a StoredCoordinateGrid2D
        keys += ["x_faces", "y_faces"]
    if kind == "focus":
        keys += ["max_mu", "spectral_index", "h0"]
    got = _run(tmp_path, kind, _inputs(data, keys))
    want = {k: data[k] for k in data if k.startswith("end_")}
    dt_rtol = 1e-12 if kind == "parker" else 1e-10
    assert "coefficient fields are not configured" in _text(got["error_unconfigured"])
    # compute_adaptive_time_step before the first step is that step's dt
    np.testing.assert_allclose(got["dts"][0], data["dts"][0], rtol=dt_rtol)
    np.testing.assert_allclose(got["dts"][1:], data["dts"], rtol=dt_rtol, atol=0)
    assert got["time_step_after"][0] == got["dts"][-1]
    _compare_state(got, want, "end", data)
    if int(data["stochastic"]):
        np.testing.assert_allclose(got["graph_dts"], data["dts"], rtol=dt_rtol, atol=0)
        for key in FIELDS:
            assert np.array_equal(got[f"graph_{key}"], got[f"end_{key}"]), key
        assert "Courant" in _text(got["error_courant"])
    # set_precision(KPT_PRECISION_MIXED): the bars of test_gpu_library_mixed.py
    # against the FP64 steps of the same classes
    np.testing.assert_allclose(got["mixed_dts"], got["dts"][1:],
                               rtol=1e-3 if kind == "focus" else 1e-5, atol=0)
    for key in ("status", "id", "w", "level", "key"):
        assert np.array_equal(got[f"mixed_{key}"], got[f"end_{key}"]), key
    wx = data["x_edges"][-1] - data["x_edges"][0]
    wy = data["y_edges"][-1] - data["y_edges"][0]
    for key, width in (("x", wx), ("y", wy)):
        d = np.abs(got[f"mixed_{key}"] - got[f"end_{key}"])
        assert (np.minimum(d, np.abs(width - d)) / width).max() <= 1e-6, key


@pytest.mark.parametrize("name", ["lib_system.npz", "lib_system_stored.npz"])
def test_cxx_particle_system_lifecycle_matches_reference(tmp_path, name):
    data = load_golden(name)
    keys = ["x_edges", "y_edges", "count", "split_ratio", "min_child_weight"]
    if "x_faces" in data:
        keys += ["x_faces", "y_faces"]
    rec = _inputs(data, keys)
    got = _run(tmp_path, "system", rec)
    for op in ("boundary", "sort", "compact", "split", "capture"):
        assert int(got[f"{op}_count"][0]) == int(data[f"{op}_count"]), op
        for key in FIELDS:
            assert np.array_equal(got[f"{op}_{key}"], data[f"{op}_{key}"]), (op, key)
    assert [int(v) for v in got["split_stats"]] == [int(v) for v in data["split_stats"]]
