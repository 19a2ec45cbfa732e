"""Generate the golden fixtures in tests/golden/ from the reference itself.

Run here (where the reference checkout exists) after ``make -C oracle ref``:

    python tests/golden/make_golden.py

Every output comes from the reference's own, unmodified driver code
(src/main.cpp and include/) compiled on the project's Kokkos-API shim
(oracle/_ref/libkpt_ref.so), with the shim's random pool drawing the keyed
Philox stream.  The fixtures store their inputs (fields, particles,
parameters) so the tests replay them without the reference: the oracle is
checked against them on the CPU and the GPU library against the oracle.

Cases
  tables_*.npz        coefficient tables (Parker 16 / focused 21 components)
                      on a uniform grid (compact reader path) and on
                      stretched y edges (StoredCoordinateGrid path)
  push_*.npz          one-interval pushes (Parker / focused, uniform /
                      stretched, adaptive and fixed dt) from injected states
  inject.npz          inject_uniform_particles with and without a y band
  split.npz           split_particles on a momentum ladder near thresholds,
                      including capacity overflow
  cli/                the reference CLI run end to end: summary.csv,
                      momentum_histogram_*.csv, particles_*.bin (v4), and a
                      restart from the frame-2 snapshot
"""
from __future__ import annotations

import importlib
import os
import shutil
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

fields = importlib.import_module("kokkos-particletransport_gb300.fields")
binding = importlib.import_module("binding")

SEED = 114514


def field_arrays(prefix: str, f) -> dict:
    return {f"{prefix}_x_edges": f.x_edges, f"{prefix}_y_edges": f.y_edges,
            f"{prefix}_b": f.b, f"{prefix}_v": f.v}


def params_arrays(params: dict) -> dict:
    return {"param_names": np.array(list(params.keys())),
            "param_values": np.array([float(v) for v in params.values()])}


def particles_arrays(prefix: str, parts: dict, count: int) -> dict:
    return {f"{prefix}_{k}": v[:count].copy() for k, v in parts.items()}


def uniform_fields():
    f0 = fields.harris_field(32, 64, noise=0.01, seed=1)
    f1 = fields.harris_field(32, 64, noise=0.01, seed=2)
    return f0, f1


def stretched_fields():
    ye = fields.stretched_edges(48, -2.0, 2.0)
    f0 = fields.harris_field(24, 48, y_edges=ye, island_amplitude=0.1, noise=0.01, seed=3)
    f1 = fields.harris_field(24, 48, y_edges=ye, island_amplitude=0.1, noise=0.01, seed=4)
    return f0, f1


def make_tables(ref, out_dir):
    with tempfile.TemporaryDirectory() as tmp:
        f0, _ = uniform_fields()
        path = fields.field_file_path(tmp, 0)
        fields.write_compact_field(path, f0)
        np.savez_compressed(os.path.join(out_dir, "tables_uniform.npz"),
                            parker=ref.table(path, False), focused=ref.table(path, True),
                            **field_arrays("field", f0))
    s0, _ = stretched_fields()
    np.savez_compressed(os.path.join(out_dir, "tables_stretched.npz"),
                        parker=ref.table_stored(s0, False), focused=ref.table_stored(s0, True),
                        **field_arrays("field", s0))


def make_inject(ref, out_dir):
    params = binding.default_params()
    cap = 3000
    with tempfile.TemporaryDirectory() as tmp:
        f0, f1 = uniform_fields()
        fields.write_compact_field(fields.field_file_path(tmp, 5), f0)
        full = binding.empty_particles(cap)
        n_full = ref.inject(tmp, params, SEED, 5, cap, 0, 1000, full)
        band = binding.empty_particles(cap)
        n_band = ref.inject(tmp, params, SEED, 5, cap, 0, 1000, band, band=(-0.2, 0.2))
        # capacity clamp: 2500 stored, 1000 requested, capacity 3000 -> 500
        clamp = binding.empty_particles(cap)
        clamp["status"][:2500] = 0
        n_clamp = ref.inject(tmp, params, SEED, 5, cap, 2500, 1000, clamp)
    np.savez_compressed(os.path.join(out_dir, "inject.npz"), frame=5, seed=SEED, capacity=cap,
                        n_full=n_full, n_band=n_band, n_clamp=n_clamp,
                        **field_arrays("field", f0), **params_arrays(params),
                        **particles_arrays("full", full, cap),
                        **particles_arrays("band", band, cap),
                        **particles_arrays("clamp", clamp, cap))


def make_push(ref, out_dir, name, focused, stretched, count, frame, overrides):
    params = binding.default_params(kperp_over_kpara=0.05, focused=int(focused), **overrides)
    cap = count
    f0, f1 = stretched_fields() if stretched else uniform_fields()
    with tempfile.TemporaryDirectory() as tmp:
        # The start state comes from the reference inject on a uniform grid of
        # the same extent (the compact reader rejects stretched edges); it is
        # stored in the fixture, so only the push depends on the grid path.
        u0, u1 = uniform_fields()
        fields.write_compact_field(fields.field_file_path(tmp, frame), f0 if not stretched else u0)
        fields.write_compact_field(fields.field_file_path(tmp, frame + 1),
                                   f1 if not stretched else u1)
        parts = binding.empty_particles(cap)
        n = ref.inject(tmp, params, SEED, frame, cap, 0, count, parts, band=(-0.3, 0.3))
        # a few particles start at the interval start, one is already inactive
        parts["t"][: n // 8] = frame * params["mhd_dt"]
        parts["status"][n - 1] = 2
        start = {k: v.copy() for k, v in parts.items()}
        if stretched:
            ref.push_stored(f0, f1, params, SEED, frame, cap, n, parts)
        else:
            ref.push(tmp, params, SEED, frame, cap, n, parts)
    np.savez_compressed(os.path.join(out_dir, f"push_{name}.npz"), frame=frame, seed=SEED,
                        count=n, **field_arrays("lower", f0), **field_arrays("upper", f1),
                        **params_arrays(params), **particles_arrays("start", start, n),
                        **particles_arrays("end", parts, n))


def make_split(ref, out_dir):
    params = binding.default_params(split_ratio=1.2, pmin_split_over_p0=2.0)
    rng = np.random.default_rng(7)
    count, cap = 600, 900
    parts = binding.empty_particles(cap)
    parts["status"][:count] = rng.choice([0, 0, 0, 1, 2], size=count).astype(np.int32)
    parts["level"][:count] = rng.integers(0, 6, size=count).astype(np.int32)
    thr = 0.2 * 1.2 ** parts["level"][:count]
    # momenta at, just above and just below the level threshold, and above pmax
    choice = rng.integers(0, 5, size=count)
    p = np.where(choice == 0, thr, np.where(choice == 1, np.nextafter(thr, np.inf),
                 np.where(choice == 2, thr * 1.05, np.where(choice == 3, thr * 0.95, 12.0))))
    parts["p"][:count] = p
    parts["x"][:count] = rng.uniform(-1, 1, count)
    parts["y"][:count] = rng.uniform(-2, 2, count)
    parts["t"][:count] = rng.uniform(0, 0.1, count)
    parts["dt"][:count] = rng.uniform(1e-6, 1e-4, count)
    parts["w"][:count] = 0.5 ** parts["level"][:count]
    parts["mu"][:count] = rng.uniform(-0.99, 0.99, count)
    start = {k: v.copy() for k, v in parts.items()}
    with tempfile.TemporaryDirectory() as tmp:
        f0, _ = uniform_fields()
        fields.write_compact_field(fields.field_file_path(tmp, 0), f0)
        n1, s1, k1 = ref.split(tmp, params, 0, cap, count, parts)
        small = {k: v.copy() for k, v in start.items()}
        n2, s2, k2 = ref.split(tmp, params, 0, count + 40, count, small)
    np.savez_compressed(os.path.join(out_dir, "split.npz"), count=count, capacity=cap,
                        small_capacity=count + 40, new_count=n1, split=s1, skipped=k1,
                        small_new_count=n2, small_split=s2, small_skipped=k2,
                        **params_arrays(params), **particles_arrays("start", start, cap),
                        **particles_arrays("end", parts, cap),
                        **particles_arrays("small_end", small, count + 40))


def make_qlt(ref, out_dir):
    """The reference's LegencyModel slab-QLT D_mumu and dD_mumu/dmu on a
    spread of inputs (including mu = 0, +-1 and the regularised edge)."""
    rng = np.random.default_rng(11)
    n = 4000
    mu = np.concatenate([rng.uniform(-1, 1, n), [0.0, -0.0, 1.0, -1.0, 0.999999, -0.999999,
                                                 1e-9, -1e-9, 1e-6, -1e-6]])
    m = mu.size
    omega = 10 ** rng.uniform(0, 4, m)
    speed = 10 ** rng.uniform(-1, 3, m)
    sigma2 = 10 ** rng.uniform(-2, 0, m)
    lc = rng.uniform(0.01, 0.2, m)
    gk = rng.uniform(1.5, 2.0, m)
    h0 = np.where(rng.uniform(size=m) < 0.5, 1e-6, 1e-3)
    d, dd = ref.qlt(mu, omega, speed, sigma2, lc, gk, h0)
    np.savez_compressed(os.path.join(out_dir, "qlt_closure.npz"), mu=mu, omega=omega,
                        speed=speed, sigma2=sigma2, lc=lc, gk=gk, h0=h0, dmumu=d, dmumu_dmu=dd)


def make_cli(ref, out_dir):
    cli_dir = os.path.join(out_dir, "cli")
    if os.path.isdir(cli_dir):
        shutil.rmtree(cli_dir)
    os.makedirs(cli_dir)
    frames = [fields.harris_field(32, 64, noise=0.01, seed=10 + k) for k in range(4)]
    arrays = {}
    for k, f in enumerate(frames):
        arrays.update(field_arrays(f"frame{k}", f))
    np.savez_compressed(os.path.join(cli_dir, "fields.npz"), **arrays)
    argv_common = ["--profile", "smoke", "--particles-per-frame", "200", "--rank-scale", "2",
                   "--capacity", "1000", "--seed", str(SEED), "--split-ratio", "1.2",
                   "--pmin-split-over-p0", "1.02", "--histogram-interval", "1",
                   "--particle-snapshot-interval", "1"]
    with tempfile.TemporaryDirectory() as tmp:
        field_dir = os.path.join(tmp, "fields")
        os.makedirs(field_dir)
        for k, f in enumerate(frames):
            fields.write_compact_field(fields.field_file_path(field_dir, k), f)
        run_dir = os.path.join(tmp, "run")
        rc = ref.main(argv_common + ["--field-dir", field_dir, "--output-dir", run_dir,
                                     "--frames", "2"], frame_base=0)
        assert rc == 0
        restart_dir = os.path.join(tmp, "restart")
        os.makedirs(restart_dir)
        shutil.copy(os.path.join(run_dir, "particles_00002.bin"), restart_dir)
        rc = ref.main(argv_common + ["--field-dir", field_dir, "--output-dir", restart_dir,
                                     "--restart-particle-snapshot",
                                     os.path.join(restart_dir, "particles_00002.bin"),
                                     "--frames", "1"], frame_base=2)
        assert rc == 0
        for sub in ("run", "restart"):
            dst = os.path.join(cli_dir, sub)
            os.makedirs(dst)
            for name in sorted(os.listdir(os.path.join(tmp, sub))):
                shutil.copy(os.path.join(tmp, sub, name), dst)
    with open(os.path.join(cli_dir, "argv.txt"), "w") as stream:
        stream.write(" ".join(argv_common) + "\n")


def main() -> None:
    ref = binding.ReferenceHarness()
    out_dir = HERE
    make_tables(ref, out_dir)
    make_inject(ref, out_dir)
    make_push(ref, out_dir, "parker_uniform", False, False, 1500, 3, {})
    make_push(ref, out_dir, "parker_fixed_dt", False, False, 600, 0,
              dict(dt_min_rel=1.0e-2, dt_max_rel=1.0e-2))
    make_push(ref, out_dir, "parker_stretched", False, True, 800, 2, {})
    make_push(ref, out_dir, "focused_uniform", True, False, 160, 3, {})
    make_push(ref, out_dir, "focused_stretched", True, True, 96, 1, {})
    make_split(ref, out_dir)
    make_qlt(ref, out_dir)
    make_cli(ref, out_dir)


if __name__ == "__main__":
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    main()
