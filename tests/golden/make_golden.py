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
  lib_parker_*.npz    the header library's ParkerSolver (stochastic and
                      deterministic steps, both diffusion branches, periodic
                      and open boundaries) on a uniform Cartesian grid
  lib_generator.npz   ParticleGenerator: region sampling with and without the
                      field threshold predicate, field and grid candidate
                      sets (indices and cumulative volumes), injection and
                      recycling from them, cell/face/mixed centred fields,
                      physical and ghosted domains
  lib_parker_coefficients.npz
                      ParkerCoefficient::make_legacy_transport_coefficient_
                      fields and the solver's packed basis: README and
                      constant-ratio branches, constant and field
                      turbulence, floors, both ghost-fill modes, open and
                      periodic axes, and two failures' messages
  lib_focus_coefficients.npz
                      FocusCoefficient::make_legacy_transport_coefficient_
                      fields[_with_time_derivative] and the focused packed
                      basis over the same variations, with and without
                      partial_t V
  lib_system.npz      ParticleSystem lifecycle: boundary conditions,
                      sort_by_key, compact_active_particles,
                      split_particles_on_energy_growth, capture_previous_positions
  lib_*_stored*.npz   the solver, lifecycle, generator and coefficient cases
                      on a StoredCoordinateGrid with stretched x and y faces

  c1/                 the strict CLI run of the 256x512 configuration
                      (summary, 128-bin histogram, first snapshot records)

``python tests/golden/make_golden.py lib`` (or ``c1``, ``stored``) regenerates
only those files.
"""
from __future__ import annotations

import importlib
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
ORACLE = os.path.join(ROOT, "oracle")
sys.path.insert(0, ORACLE)

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


C1_ARGV = ["--profile", "smoke", "--frames", "1", "--particles-per-frame", "1600",
           "--rank-scale", "16", "--capacity", "65536", "--overwrite-output"]


def make_c1(ref, out_dir):
    """The strict CLI run of the 256x512 configuration: Harris sheet with the
    default parameters, no islands, no noise, identical frames 0 and 1;
    25,600 particles.  Kept: summary.csv, the 128-bin histogram and the first
    2048 snapshot records (the snapshot itself is 2.5 MB)."""
    formats = importlib.import_module("kokkos-particletransport_gb300.formats")
    c1_dir = os.path.join(out_dir, "c1")
    if os.path.isdir(c1_dir):
        shutil.rmtree(c1_dir)
    os.makedirs(c1_dir)
    field = fields.harris_field(256, 512)
    with tempfile.TemporaryDirectory() as tmp:
        field_dir = os.path.join(tmp, "fields")
        os.makedirs(field_dir)
        for k in range(2):
            fields.write_compact_field(fields.field_file_path(field_dir, k), field)
        run_dir = os.path.join(tmp, "run")
        rc = ref.main(C1_ARGV + ["--field-dir", field_dir, "--output-dir", run_dir],
                      frame_base=0)
        assert rc == 0
        for name in ("summary.csv", "momentum_histogram_00001.csv"):
            shutil.copy(os.path.join(run_dir, name), c1_dir)
        snap = formats.read_snapshot(os.path.join(run_dir, "particles_00001.bin"))
        head = snap.records[:2048]
        np.savez_compressed(os.path.join(c1_dir, "snapshot_head.npz"), count=snap.count,
                            capacity=snap.capacity,
                            **{name: head[name] for name in head.dtype.names})
    with open(os.path.join(c1_dir, "argv.txt"), "w") as stream:
        stream.write(" ".join(C1_ARGV) + "\n")


lib_basis = fields.library_parker_basis
lib_focus_basis = fields.library_focus_basis


def lib_population(rng, count: int, capacity: int, x_edges, y_edges, open_y: bool) -> dict:
    system = binding.lib_default_system(count, capacity)
    system["x"][:count] = rng.uniform(x_edges[0], x_edges[-1], count)
    lo, hi = y_edges[0], y_edges[-1]
    if open_y:
        hi_band = hi - 0.02 * (hi - lo)
        system["y"][:count] = rng.uniform(lo, hi, count)
        system["y"][:count:7] = rng.uniform(hi_band, hi, len(system["y"][:count:7]))
    else:
        system["y"][:count] = rng.uniform(lo, hi, count)
    system["prev_x"][:count] = system["x"][:count] - 0.01
    system["prev_y"][:count] = system["y"][:count] + 0.01
    system["p"][:count] = np.exp(rng.uniform(np.log(0.05), np.log(3.0), count))
    system["mu"][:count] = rng.uniform(-1, 1, count)
    system["status"][:count:13] = 2  # a few inactive particles inside the count
    return system


def lib_save(out_dir, name, **arrays):
    np.savez_compressed(os.path.join(out_dir, name), **arrays)


class LibGeometry:
    """Axes of a library grid: uniform edges (the analytic grid), or
    stretched edges whose n + 5 faces (two ghost faces per side, continued
    periodically) make a StoredCoordinateGrid.  The stored files carry the
    faces, the tests build the same grid from them."""

    def __init__(self, nx, ny, xlim, ylim, stored):
        self.nx, self.ny, self.stored = nx, ny, stored
        if stored:
            self.xe = fields.stretched_edges(nx, xlim[0], xlim[1], strength=1.5)
            self.ye = fields.stretched_edges(ny, ylim[0], ylim[1], strength=4.0)
            self.xf = fields.ghosted_faces(self.xe)
            self.yf = fields.ghosted_faces(self.ye)
        else:
            self.xe = np.linspace(xlim[0], xlim[1], nx + 1)
            self.ye = np.linspace(ylim[0], ylim[1], ny + 1)

    @property
    def suffix(self):
        return "_stored" if self.stored else ""

    def grid(self, periodic):
        g = dict(x_edges=self.xe, y_edges=self.ye, periodic=np.array(periodic, dtype=np.int32))
        g.update(self.extra())
        return g

    def extra(self):
        return dict(x_faces=self.xf, y_faces=self.yf) if self.stored else {}

    def centres(self):
        """Ghosted cell centres (n + 4) of each axis; None on the uniform
        grid, whose helpers form them from the spacing."""
        if not self.stored:
            return None
        return fields.cell_centres(self.xf), fields.cell_centres(self.yf)


def make_lib(ref, out_dir, stored=False):
    rng = np.random.default_rng(2718 + (1 if stored else 0))
    nx, ny = 24, 40
    geo = LibGeometry(nx, ny, (-1.0, 1.0), (-2.0, 2.0), stored)
    xe, ye = geo.xe, geo.ye
    props = dict(rest_mass=1.0, charge=1.0, speed_of_light=1.0, energy_scale=1.0, courant=0.3)
    cases = (("readme_periodic", True, (1, 1), True, 4),
             ("ratio_open", False, (1, 0), True, 4),
             ("readme_deterministic", True, (1, 0), False, 3))
    for name, readme, periodic, stochastic, steps in cases:
        grid = geo.grid(periodic)
        basis = lib_basis(nx, ny, xe, ye, readme, centres=geo.centres())
        count, capacity = 700, 768
        start = lib_population(rng, count, capacity, xe, ye, periodic[1] == 0)
        system = {k: v.copy() for k, v in start.items()}
        dts = ref.lib_parker(grid, basis, not readme, props, SEED, 10, steps, stochastic, count,
                             system)
        lib_save(out_dir, f"lib_parker{geo.suffix}_{name}.npz", x_edges=xe, y_edges=ye,
                 **geo.extra(),
                 periodic=grid["periodic"], basis=basis, constant_ratio=int(not readme),
                 stochastic=int(stochastic), steps=steps, first_step=10, seed=SEED,
                 count=count, courant=props["courant"], dts=dts,
                 **{f"start_{k}": v for k, v in start.items()},
                 **{f"end_{k}": v for k, v in system.items()})
    # FocusTransportSolver
    focus_cases = (("readme_periodic", False, (1, 1), True, 4, 1.0),
                   ("ratio_open_mumax", True, (1, 0), True, 3, 0.95),
                   ("deterministic", False, (1, 1), False, 3, 1.0))
    scattering = dict(spectral_index=5.0 / 3.0, h0=1e-6)
    for name, ratio, periodic, stochastic, steps, max_mu in focus_cases:
        grid = geo.grid(periodic)
        basis = lib_focus_basis(nx, ny, xe, ye, centres=geo.centres())
        count, capacity = 600, 640
        start = lib_population(rng, count, capacity, xe, ye, periodic[1] == 0)
        system = {k: v.copy() for k, v in start.items()}
        scat = dict(scattering, max_mu=max_mu)
        dts = ref.lib_focus(grid, basis, ratio, props, scat, SEED, 20, steps, stochastic, count,
                            system)
        lib_save(out_dir, f"lib_focus{geo.suffix}_{name}.npz", x_edges=xe, y_edges=ye,
                 **geo.extra(),
                 periodic=grid["periodic"], basis=basis, constant_ratio=int(ratio),
                 stochastic=int(stochastic), steps=steps, first_step=20, seed=SEED,
                 count=count, courant=props["courant"], dts=dts,
                 spectral_index=scattering["spectral_index"], h0=scattering["h0"],
                 max_mu=max_mu,
                 **{f"start_{k}": v for k, v in start.items()},
                 **{f"end_{k}": v for k, v in system.items()})
    # injected noise: caller normals [steps][4][count] replace the random pool's
    # draws on both sides; a tenth of them widened fourfold to reach the
    # pitch-angle clamp and the open boundaries
    nrng = np.random.default_rng(31415)
    for kind, periodic, steps in () if stored else (("parker", (1, 0), 3), ("focus", (1, 0), 3)):
        grid = dict(x_edges=xe, y_edges=ye, periodic=np.array(periodic, dtype=np.int32))
        count, capacity = 500, 512
        start = lib_population(nrng, count, capacity, xe, ye, True)
        system = {k: v.copy() for k, v in start.items()}
        normals = nrng.standard_normal((steps, 4, count))
        normals[nrng.random(normals.shape) < 0.1] *= 4.0
        if kind == "parker":
            basis = lib_basis(nx, ny, xe, ye, True)
            dts = ref.lib_parker(grid, basis, False, props, SEED, 0, steps, True, count, system,
                                 normals)
            extra = dict(constant_ratio=0)
        else:
            basis = lib_focus_basis(nx, ny, xe, ye)
            dts = ref.lib_focus(grid, basis, False, props, dict(scattering, max_mu=0.97), SEED,
                                0, steps, True, count, system, normals)
            extra = dict(constant_ratio=0, spectral_index=scattering["spectral_index"],
                         h0=scattering["h0"], max_mu=0.97)
        lib_save(out_dir, f"lib_noise_{kind}.npz", x_edges=xe, y_edges=ye,
                 periodic=grid["periodic"], basis=basis, steps=steps, count=count,
                 courant=props["courant"], dts=dts, normals=normals, **extra,
                 **{f"start_{k}": v for k, v in start.items()},
                 **{f"end_{k}": v for k, v in system.items()})
    # ParticleSystem lifecycle
    grid = geo.grid((1, 0))
    props_sys = dict(props, split_ratio=2.0, min_child_weight=0.2)
    arrays = {}
    count, capacity = 500, 560
    base = lib_population(rng, count, capacity, xe, ye, True)
    base["x"][:count:5] += 2.5  # outside the periodic x range
    base["y"][:count:9] = 2.1   # outside the open y range
    base["key"][:count] = rng.integers(-3, 41, count)
    base["w"][:count] = 2.0 ** -rng.integers(0, 4, count)
    # baselines: valid for most, zero for a few; momenta spread energy ratios
    ke = np.sqrt(1.0 + base["p"] ** 2) - 1.0
    base["e0"][:count] = ke[:count] / np.exp(rng.uniform(0.0, np.log(20.0), count))
    base["e0"][:count:11] = 0.0
    base["level"][:count] = rng.integers(0, 3, count)
    for op, key_range in (("boundary", (0, 0)), ("sort", (-3, 40)), ("compact", (0, 0)),
                          ("split", (0, 0)), ("capture", (0, 0))):
        system = {k: v.copy() for k, v in base.items()}
        new_count, stats = ref.lib_system(grid, props_sys, op, count, system, key_range)
        arrays[f"{op}_count"] = new_count
        arrays[f"{op}_stats"] = np.array(stats, dtype=np.uint64)
        for k, v in system.items():
            arrays[f"{op}_{k}"] = v
    for k, v in base.items():
        arrays[f"start_{k}"] = v
    lib_save(out_dir, f"lib_system{geo.suffix}.npz", x_edges=xe, y_edges=ye,
             periodic=grid["periodic"], **geo.extra(),
             count=count, split_ratio=props_sys["split_ratio"],
             min_child_weight=props_sys["min_child_weight"], **arrays)


def generator_fields(nx: int, ny: int, x_edges, y_edges, geo=None) -> dict:
    """Fields of the ParticleGenerator cases, in the Field's stored order
    (dim 0 fastest over the ghosted extent of the centering), at the cell
    centres and faces of the uniform grid or of `geo`'s stored one."""
    dx = (x_edges[-1] - x_edges[0]) / nx
    dy = (y_edges[-1] - y_edges[0]) / ny

    def coords(n, x0, d, face):
        k = np.arange(n + 4 + int(face)) - 2.0
        return x0 + (k if face else k + 0.5) * d

    if geo is not None and geo.stored:
        (xc, yc), xf, yf = geo.centres(), geo.xf, geo.yf
    else:
        xc, yc = coords(nx, x_edges[0], dx, False), coords(ny, y_edges[0], dy, False)
        xf, yf = coords(nx, x_edges[0], dx, True), coords(ny, y_edges[0], dy, True)
    scalar_cell = (np.cos(2.0 * xc)[None, :] * np.exp(-yc[:, None] ** 2)).ravel()
    vec_face = np.stack([np.sin(3.0 * xf)[None, :] + 0.0 * yf[:, None],
                         np.tanh(yf[:, None] / 0.4) * np.cos(xf)[None, :],
                         xf[None, :] * yf[:, None]], axis=-1).reshape(-1, 3)
    mixed = (np.sin(xc)[None, :] * yf[:, None]).ravel()
    return {"scalar_cell": (scalar_cell, (0, 0)), "vec_face": (vec_face, (1, 1)),
            "mixed": (mixed, (0, 1))}


# op, field, region (None = grid domain), predicate (threshold, comparison,
# component, domain), kinematics (p, mu, weight, status), plan (first index,
# count, first id, attempts), selection, population
GENERATOR_CASES = (
    ("inject_uniform", "inject_uniform", "scalar_cell", (-1.0, -1.5, 1.5, 1.0),
     (0.0, 1, 0, 0), (0.7, -0.3, 2.0, 0), (0, 500, 0, 64), 0, "empty"),
    ("inject_uniform_if", "inject_uniform_if", "scalar_cell", (-1.3, -2.0, 2.1, 2.0),
     (0.2, 0, 0, 0), (1.1, 0.5, 1.0, 0), (120, 400, 9000, 4), 0, "partial"),
    ("inject_if_face_ghosted", "inject_uniform_if", "vec_face", (-1.5, -2.2, 2.3, 2.2),
     (0.5, 4, 1, 1), (0.3, 0.0, 0.5, 0), (0, 300, 5, 16), 0, "empty"),
    ("inject_where_field_region", "inject_where_field", "scalar_cell", (-0.8, -1.0, 1.2, 1.5),
     (0.1, 1, 0, 0), (0.9, 0.1, 1.0, 0), (120, 600, 120, 64), 0, "partial"),
    ("inject_where_field_whole", "inject_where_field", "vec_face", None,
     (0.4, 5, 2, 0), (2.0, -0.9, 1.0, 1), (0, 500, 0, 64), 0, "empty"),
    ("inject_where_field_mixed", "inject_where_field", "mixed", None,
     (0.3, 0, 0, 1), (0.2, 0.2, 3.0, 0), (0, 400, 77, 64), 0, "empty"),
    ("inject_in_grid", "inject_in_grid", "scalar_cell", None,
     (0.0, 1, 0, 0), (0.5, 0.0, 1.0, 0), (0, 700, 0, 64), 0, "empty"),
    ("inject_in_grid_ghosted", "inject_in_grid", "scalar_cell", None,
     (0.0, 1, 0, 1), (0.5, 0.4, 1.0, 0), (120, 300, 1000, 64), 0, "partial"),
    ("recycle_uniform_escaped", "recycle_uniform", "scalar_cell", (-1.0, -1.0, 1.0, 1.0),
     (0.0, 1, 0, 0), (0.8, 0.0, 1.0, 0), (0, 0, 0, 64), 0, "mixed"),
    ("recycle_uniform_if_recyclable", "recycle_uniform_if", "scalar_cell",
     (-1.3, -2.0, 2.1, 2.0), (0.3, 0, 0, 0), (0.6, 0.2, 1.5, 0), (0, 0, 0, 3), 2, "mixed"),
    ("recycle_where_field_inactive", "recycle_where_field", "vec_face", (-1.0, -1.5, 1.0, 1.5),
     (0.2, 2, 0, 0), (1.2, -0.5, 1.0, 0), (0, 0, 0, 64), 1, "mixed"),
    ("recycle_where_field_whole", "recycle_where_field", "mixed", None,
     (-0.1, 3, 0, 0), (0.4, 0.0, 1.0, 0), (0, 0, 0, 64), 2, "mixed"),
    ("recycle_in_grid", "recycle_in_grid", "scalar_cell", None,
     (0.0, 1, 0, 0), (0.7, 0.3, 1.0, 0), (0, 0, 0, 64), 2, "mixed"),
)

# field, region, predicate (threshold, comparison, component, domain); field
# None = the grid's cells
CANDIDATE_CASES = (
    ("field_cell_region", "scalar_cell", (-0.8, -1.0, 1.2, 1.5), (0.1, 1, 0, 0)),
    ("field_face_ghosted", "vec_face", None, (0.4, 5, 2, 1)),
    ("field_mixed", "mixed", None, (0.3, 0, 0, 0)),
    ("grid_physical", None, None, (0.0, 0, 0, 0)),
    ("grid_ghosted", None, None, (0.0, 0, 0, 1)),
)


def make_generator(ref, out_dir, stored=False):
    """ParticleGenerator cases from the reference's own templates."""
    rng = np.random.default_rng(1618 + (1 if stored else 0))
    nx, ny = 24, 40
    geo = LibGeometry(nx, ny, (-1.3, 2.1), (-2.0, 2.0), stored)
    xe, ye = geo.xe, geo.ye
    grid = geo.grid((1, 0))
    props = dict(rest_mass=1.0, charge=1.0, speed_of_light=1.0, energy_scale=1.0)
    fields = generator_fields(nx, ny, xe, ye, geo)
    arrays = {f"field_{name}": values for name, (values, _) in fields.items()}
    for name, (_, cent) in fields.items():
        arrays[f"centering_{name}"] = np.array(cent, dtype=np.int32)
    capacity = 1024
    for k, (name, op, field, region, pred, kin, plan, selection, population) in enumerate(
            GENERATOR_CASES):
        count = {"empty": 0, "partial": 120, "mixed": 900}[population]
        start = lib_population(rng, count, capacity, xe, ye, True) if count else \
            binding.lib_default_system(0, capacity)
        if population == "mixed":
            start["status"][:count] = rng.choice([0, 1, 2], count, p=[0.4, 0.35, 0.25])
        system = {key: v.copy() for key, v in start.items()}
        values, cent = fields[field]
        predicate = dict(threshold=pred[0], comparison=pred[1], component=pred[2],
                         domain=pred[3])
        seed, frame = SEED + k, 3 + k
        end_count = ref.lib_generator(grid, props, op, count, system, field=values,
                                      centering=cent, region=region, predicate=predicate,
                                      kinematics=kin, plan=plan, selection=selection, seed=seed,
                                      frame=frame)
        arrays[f"{name}_case"] = np.array(
            [k, count, end_count, selection, seed, frame], dtype=np.int64)
        arrays[f"{name}_op"] = np.array(op)
        arrays[f"{name}_field"] = np.array(field)
        arrays[f"{name}_region"] = np.array(region if region is not None else [np.nan] * 4)
        arrays[f"{name}_predicate"] = np.array(pred, dtype=np.float64)
        arrays[f"{name}_kinematics"] = np.array(kin, dtype=np.float64)
        arrays[f"{name}_plan"] = np.array(plan, dtype=np.uint64)
        for key, v in start.items():
            arrays[f"{name}_start_{key}"] = v
        for key, v in system.items():
            arrays[f"{name}_end_{key}"] = v
    for name, field, region, pred in CANDIDATE_CASES:
        predicate = dict(threshold=pred[0], comparison=pred[1], component=pred[2],
                         domain=pred[3])
        if field is None:
            idx, cum, total = ref.lib_candidates(grid, "grid", predicate=predicate)
        else:
            values, cent = fields[field]
            idx, cum, total = ref.lib_candidates(grid, "field", field=values, centering=cent,
                                                 region=region, predicate=predicate)
        arrays[f"cand_{name}_indices"] = idx
        arrays[f"cand_{name}_cumulative"] = cum
        arrays[f"cand_{name}_total"] = np.array(total)
        arrays[f"cand_{name}_field"] = np.array(field if field is not None else "")
        arrays[f"cand_{name}_region"] = np.array(region if region is not None else [np.nan] * 4)
        arrays[f"cand_{name}_predicate"] = np.array(pred, dtype=np.float64)
    lib_save(out_dir, f"lib_generator{geo.suffix}.npz", x_edges=xe, y_edges=ye,
             periodic=grid["periodic"], **geo.extra(),
             cases=np.array([c[0] for c in GENERATOR_CASES]),
             candidate_cases=np.array([c[0] for c in CANDIDATE_CASES]), **arrays)


def coefficient_inputs(nx: int, ny: int, x_edges, y_edges, variant: int, centres=None):
    """Cell-centred B and V over the ghosted cells (x fastest), analytic
    everywhere (the caller's ghost values), plus turbulence fields; at the
    uniform grid's centres or the given (xc, yc) of a stored one."""
    dx = (x_edges[-1] - x_edges[0]) / nx
    dy = (y_edges[-1] - y_edges[0]) / ny
    xc = x_edges[0] + (np.arange(nx + 4) - 1.5) * dx
    yc = y_edges[0] + (np.arange(ny + 4) - 1.5) * dy
    if centres is not None:
        xc, yc = centres
    X, Y = np.meshgrid(xc, yc)
    bz = 0.3 + 0.1 * variant * np.cos(X + Y)
    b = np.stack([np.tanh(Y / 0.5) + 0.05 * np.sin(3 * X), 0.2 * np.sin(X) + 0.1 * variant,
                  bz], axis=-1).reshape(-1, 3)
    v = np.stack([1.0 + 0.1 * np.cos(X), 0.2 * np.sin(Y), 0.05 * variant * X],
                 axis=-1).reshape(-1, 3)
    fields = (0.3 + 0.1 * np.cos(2 * X) * np.exp(-Y ** 2),   # sigma2
              0.8 + 0.3 * np.abs(np.sin(Y)),                # l2d
              1.2 + 0.2 * X ** 2,                           # lslab
              0.9 + 0.1 * np.cos(X * Y))                    # lc
    return b, v, [f.ravel() for f in fields]


# name, periodic, variant, turbulence ("constant" or "fields"), params,
# charge, drift floor, ghost mode
COEFFICIENT_CASES = (
    ("readme_constant", (1, 0), 0, "constant", dict(), 1.0, 0.0, 0),
    ("ratio_floors", (1, 0), 1, "constant",
     dict(model=1, ratio=0.05, minimum_b=0.25, minimum_vsw=0.9, minimum_sigma2=0.4), -2.0,
     1e-3, 0),
    ("readme_fields_periodic_only", (0, 1), 2, "fields",
     dict(parallel_prefactor=1.5, perpendicular_prefactor=0.25), 1.0, 0.0, 1),
    ("ratio_fields_open", (0, 0), 1, "fields", dict(model=1, ratio=0.3), 0.5, 0.0, 0),
)


def make_parker_coefficients(ref, out_dir, stored=False):
    """The reference's Parker coefficient precompute and packed basis."""
    nx, ny = 20, 28
    geo = LibGeometry(nx, ny, (-1.3, 2.1), (-2.0, 2.0), stored)
    xe, ye = geo.xe, geo.ye
    arrays = {}
    for name, periodic, variant, turb, params, charge, floor, ghost in COEFFICIENT_CASES:
        grid = geo.grid(periodic)
        b, v, fields = coefficient_inputs(nx, ny, xe, ye, variant, geo.centres())
        constant = (0.35, 0.9, 1.4, -1.0 if variant == 0 else 1.1)
        props = dict(rest_mass=1.0, charge=charge, speed_of_light=1.0)
        packed = ref.lib_parker_coefficients(
            grid, b, v, turbulence=constant,
            turbulence_fields=fields if turb == "fields" else None, props=props,
            params=params, drift_floor=floor, ghost_mode=ghost)
        arrays[f"{name}_periodic"] = grid["periodic"]
        arrays[f"{name}_b"] = b
        arrays[f"{name}_v"] = v
        arrays[f"{name}_turbulence"] = np.array(constant)
        arrays[f"{name}_fields"] = np.stack(fields) if turb == "fields" else np.zeros((0,))
        arrays[f"{name}_params"] = np.array(
            [params.get("model", 0), params.get("parallel_prefactor", 1.622),
             params.get("perpendicular_prefactor", 0.198), params.get("ratio", 0.0),
             params.get("minimum_b", 0.0), params.get("minimum_vsw", 0.0),
             params.get("minimum_sigma2", 0.0), floor, ghost, charge])
        arrays[f"{name}_packed"] = packed
    if stored:
        lib_save(out_dir, "lib_parker_coefficients_stored.npz", x_edges=xe, y_edges=ye,
                 **geo.extra(), cases=np.array([c[0] for c in COEFFICIENT_CASES]), **arrays)
        return
    # failures: the reference's messages
    grid = dict(x_edges=xe, y_edges=ye, periodic=np.array((1, 0), dtype=np.int32))
    errors = []
    b, v, fields = coefficient_inputs(nx, ny, xe, ye, 0)
    zero_b = b.copy()
    zero_b[(nx + 4) * 10 + 7] = 0.0
    bad_lc = [f.copy() for f in fields]
    bad_lc[3][(nx + 4) * 12 + 9] = -1.0
    # Kokkos::abort ends the process, so each failure runs in a child
    # that reports the shim's abort message
    with tempfile.TemporaryDirectory() as tmp:
        for label, b_in, turb_fields in (("zero_b", zero_b, None),
                                         ("negative_lc", b, bad_lc)):
            path = os.path.join(tmp, f"{label}.npz")
            np.savez(path, b=b_in, v=v, xe=xe, ye=ye,
                     fields=np.stack(turb_fields) if turb_fields is not None else np.zeros(0))
            code = (
                "import sys, numpy as np; sys.path.insert(0, %r); import binding\n"
                "d = np.load(%r); f = d['fields']\n"
                "grid = dict(x_edges=d['xe'], y_edges=d['ye'], periodic=np.array((1, 0)))\n"
                "binding.ReferenceHarness().lib_parker_coefficients(grid, d['b'], d['v'], "
                "turbulence_fields=list(f) if f.size else None)\n" % (ORACLE, path))
            proc = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True)
            message = ""
            for line in proc.stderr.splitlines():
                if line.startswith("Kokkos shim abort: "):
                    message = line[len("Kokkos shim abort: "):].strip()
            errors.append((label, message))
    arrays["error_names"] = np.array([e[0] for e in errors])
    arrays["error_messages"] = np.array([e[1] for e in errors])
    arrays["error_zero_b"] = zero_b
    arrays["error_negative_lc"] = np.stack(bad_lc)
    arrays["error_b"] = b
    arrays["error_v"] = v
    lib_save(out_dir, "lib_parker_coefficients.npz", x_edges=xe, y_edges=ye,
             cases=np.array([c[0] for c in COEFFICIENT_CASES]), **arrays)


# name, periodic, variant, turbulence, params, charge, builder floor, ghost
# mode, with dV/dt
FOCUS_COEFFICIENT_CASES = (
    ("readme_constant", (1, 0), 0, "constant", dict(), 1.0, 0.0, 0, False),
    ("ratio_floors_dvdt", (1, 0), 1, "constant",
     dict(model=1, ratio=0.05, minimum_b=0.25, minimum_vsw=0.9, minimum_sigma2=0.4), -2.0,
     0.05, 0, True),
    ("readme_fields_periodic_only", (0, 1), 2, "fields",
     dict(parallel_prefactor=1.5, perpendicular_prefactor=0.25), 1.0, 0.0, 1, True),
    ("ratio_fields_open", (0, 0), 1, "fields", dict(model=1, ratio=0.3), 0.5, 0.0, 0, False),
)


def make_focus_coefficients(ref, out_dir, stored=False):
    """The reference's focused coefficient precompute and packed basis."""
    nx, ny = 20, 28
    geo = LibGeometry(nx, ny, (-1.3, 2.1), (-2.0, 2.0), stored)
    xe, ye = geo.xe, geo.ye
    arrays = {}
    for (name, periodic, variant, turb, params, charge, floor, ghost,
         with_dvdt) in FOCUS_COEFFICIENT_CASES:
        grid = geo.grid(periodic)
        b, v, fields = coefficient_inputs(nx, ny, xe, ye, variant, geo.centres())
        dvdt = None
        if with_dvdt:
            dvdt = np.stack([np.cos(v[:, 0]), 0.3 * v[:, 1], 0.1 + 0.0 * v[:, 2]], axis=-1)
        constant = (0.35, 0.9, 1.4, -1.0 if variant == 0 else 1.1)
        props = dict(rest_mass=1.0, charge=charge, speed_of_light=1.0)
        packed = ref.lib_focus_coefficients(
            grid, b, v, dvdt, turbulence=constant,
            turbulence_fields=fields if turb == "fields" else None, props=props,
            params=params, builder_floor=floor, ghost_mode=ghost)
        arrays[f"{name}_periodic"] = grid["periodic"]
        arrays[f"{name}_b"] = b
        arrays[f"{name}_v"] = v
        arrays[f"{name}_dvdt"] = dvdt if dvdt is not None else np.zeros((0,))
        arrays[f"{name}_turbulence"] = np.array(constant)
        arrays[f"{name}_fields"] = np.stack(fields) if turb == "fields" else np.zeros((0,))
        arrays[f"{name}_params"] = np.array(
            [params.get("model", 0), params.get("parallel_prefactor", 1.622),
             params.get("perpendicular_prefactor", 0.198), params.get("ratio", 0.0),
             params.get("minimum_b", 0.0), params.get("minimum_vsw", 0.0),
             params.get("minimum_sigma2", 0.0), floor, ghost, charge])
        arrays[f"{name}_packed"] = packed
    lib_save(out_dir, f"lib_focus_coefficients{geo.suffix}.npz", x_edges=xe, y_edges=ye,
             **geo.extra(), cases=np.array([c[0] for c in FOCUS_COEFFICIENT_CASES]), **arrays)


def make_stored(ref, out_dir):
    """The library cases again on stored (explicit, stretched) grids:
    lib_parker_stored_*, lib_focus_stored_*, lib_system_stored,
    lib_generator_stored, lib_*_coefficients_stored."""
    make_lib(ref, out_dir, stored=True)
    make_generator(ref, out_dir, stored=True)
    make_parker_coefficients(ref, out_dir, stored=True)
    make_focus_coefficients(ref, out_dir, stored=True)


def main() -> None:
    ref = binding.ReferenceHarness()
    out_dir = HERE
    if sys.argv[1:] == ["c1"]:
        make_c1(ref, out_dir)
        return
    if sys.argv[1:] == ["generator"]:
        make_generator(ref, out_dir)
        return
    if sys.argv[1:] == ["coefficients"]:
        make_parker_coefficients(ref, out_dir)
        make_focus_coefficients(ref, out_dir)
        return
    if sys.argv[1:] == ["stored"]:
        make_stored(ref, out_dir)
        return
    make_lib(ref, out_dir)
    make_generator(ref, out_dir)
    make_parker_coefficients(ref, out_dir)
    make_focus_coefficients(ref, out_dir)
    make_stored(ref, out_dir)
    if sys.argv[1:] == ["lib"]:
        return
    make_c1(ref, out_dir)
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
