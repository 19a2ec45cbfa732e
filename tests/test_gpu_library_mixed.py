"""The mixed-precision library step against the FP64 step.

The mixed step (kpt_*_solver_set_precision(KPT_PRECISION_MIXED)) samples an
FP32 copy of the packed basis and forms the terms, the local dt bounds, the
Box-Muller noise (from the high word of each keyed draw) and, for the focused
solver, the slab-QLT pitch-angle update in FP32; positions, momenta, the
global dt and the boundary decisions stay FP64.  From the golden start states
(uniform and stored grids) and the same keyed stream, every step of the mixed
solver is compared with the FP64 solver's (itself pinned to the reference's
templates in test_gpu_library.py):

* the global dt of every step within DT_REL relative (Parker) or
  DT_REL_FOCUS (focused: the lockstep dt is set by the pitch-angle limiters,
  0.1 / |dmu/dt| and D / (dmu/dt)^2, whose rates near mu = 0 are steep in mu);
* positions within POS_REL of the periodic width, momenta within P_REL
  relative, pitch cosines within MU_ABS;
* statuses (escapes at open boundaries) identical.

A longer run (64 steps of 20 000 particles on the 1024 x 2048 library grid of
the bench): Parker keeps the paired bars on 99.9 % of the particles.  A
focused run does not stay paired that long: a particle whose pitch cosine
passes close to 0 meets the steep closure there (D' grows as |mu|^(gk-2)),
and a difference of 1e-6 in mu moves its pitch-angle dt bound, which can set
the global dt of that step, by tens of percent; FP64 runs react alike to any
perturbation.  The focused run is judged by what it computes: the time it
advances (within 1 %) and the paired momentum and pitch-cosine distributions
(16 bins each, L1 within 1 %).
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import lib_grid, load_golden

pytestmark = pytest.mark.gpu

FIELDS = ("x", "y", "prev_x", "prev_y", "prevstep_x", "prevstep_y", "p", "mu", "w", "e0",
          "status", "level", "key", "id")
DT_REL = 1e-5
DT_REL_FOCUS = 1e-3
POS_REL = 1e-6
P_REL = 1e-5
MU_ABS = 1e-4


def _state(data, prefix):
    return {k: data[f"{prefix}_{k}"].copy() for k in FIELDS}


def _run(ctx, kpt, data, focused, precision):
    grid = lib_grid(ctx, data)
    start = _state(data, "start")
    system = ctx.system(int(data["count"]), start["x"].size)
    system.upload(start)
    if focused:
        solver = ctx.focus_solver(grid, data["basis"], bool(data["constant_ratio"]),
                                  float(data["courant"]), float(data["spectral_index"]),
                                  float(data["h0"]), maximum_mu=float(data["max_mu"]))
    else:
        solver = ctx.parker_solver(grid, data["basis"], bool(data["constant_ratio"]),
                                   float(data["courant"]))
    solver.set_precision(precision)
    steps, first, seed = int(data["steps"]), int(data["first_step"]), int(data["seed"])
    dts = []
    for k in range(steps):
        if int(data["stochastic"]):
            dts.append(solver.advance_stochastic(system, seed, first + k))
        else:
            dts.append(solver.advance_deterministic(system))
    out = system.download()
    for h in (solver, system, grid):
        h.close()
    return np.array(dts), out


def _deviation(mixed, ref, width_x, width_y):
    dev = {}
    for key, width in (("x", width_x), ("y", width_y)):
        d = np.abs(mixed[key] - ref[key])
        dev[key] = np.minimum(d, np.abs(width - d)) / width
    dev["p"] = np.abs(mixed["p"] - ref["p"]) / np.maximum(np.abs(ref["p"]), 1e-300)
    dev["mu"] = np.abs(mixed["mu"] - ref["mu"])
    return dev


CASES = [("parker", c) for c in ("readme_periodic", "ratio_open", "readme_deterministic",
                                 "stored_readme_periodic", "stored_ratio_open")] + \
        [("focus", c) for c in ("readme_periodic", "ratio_open_mumax", "deterministic",
                                "stored_ratio_open_mumax")]


@pytest.mark.parametrize("kind,case", CASES)
def test_mixed_steps_track_fp64_steps(ctx, kpt, kind, case):
    data = load_golden(f"lib_{kind}_{case}.npz")
    focused = kind == "focus"
    dts64, ref = _run(ctx, kpt, data, focused, kpt.PRECISION_F64)
    dts32, mixed = _run(ctx, kpt, data, focused, kpt.PRECISION_MIXED)
    dt_dev = np.abs(dts32 / dts64 - 1.0)
    width_x = data["x_edges"][-1] - data["x_edges"][0]
    width_y = data["y_edges"][-1] - data["y_edges"][0]
    dev = _deviation(mixed, ref, width_x, width_y)
    print(kind, case, "dt", dt_dev.max(), {k: float(v.max()) for k, v in dev.items()})
    assert dt_dev.max() <= (DT_REL_FOCUS if focused else DT_REL)
    assert np.array_equal(mixed["status"], ref["status"])
    for key in ("id", "w", "level", "key", "e0"):
        assert np.array_equal(mixed[key], ref[key]), key
    assert dev["x"].max() <= POS_REL and dev["y"].max() <= POS_REL
    assert dev["p"].max() <= P_REL
    if focused:
        assert dev["mu"].max() <= MU_ABS
    else:
        assert np.array_equal(mixed["mu"], ref["mu"])


@pytest.mark.parametrize("focused", [False, True])
def test_mixed_steps_over_a_long_run(ctx, kpt, fields_mod, focused):
    nx, ny, n, steps = 1024, 2048, 20000, 64
    xe = np.linspace(-1.0, 1.0, nx + 1)
    ye = np.linspace(-2.0, 2.0, ny + 1)
    basis = (fields_mod.library_focus_basis(nx, ny, xe, ye) if focused
             else fields_mod.library_parker_basis(nx, ny, xe, ye, True))
    rng = np.random.default_rng(17)
    state = {"id": np.arange(n, dtype=np.uint64)}
    for key in kpt.SYSTEM_DOUBLE_FIELDS:
        state[key] = np.zeros(n)
    for key in kpt.SYSTEM_INT_FIELDS:
        state[key] = np.zeros(n, dtype=np.int32)
    state["x"] = rng.uniform(xe[0], xe[-1], n)
    state["y"] = rng.uniform(ye[0], ye[-1], n)
    state["p"] = np.exp(rng.uniform(np.log(0.05), np.log(3.0), n))
    state["mu"] = rng.uniform(-1.0, 1.0, n)
    state["w"] = np.ones(n)
    runs = {}
    for precision in (kpt.PRECISION_F64, kpt.PRECISION_MIXED):
        grid = ctx.grid(xe, ye, (1, 1))
        solver = (ctx.focus_solver(grid, basis, False, 0.3) if focused
                  else ctx.parker_solver(grid, basis, False, 0.3))
        solver.set_precision(precision)
        system = ctx.system(n, n)
        system.upload(state)
        dts = solver.advance_stochastic_steps(system, 5, 0, steps)
        runs[precision] = (np.asarray(dts), system.download())
        for h in (solver, system, grid):
            h.close()
    (d64, ref), (d32, mixed) = runs[kpt.PRECISION_F64], runs[kpt.PRECISION_MIXED]
    dev = _deviation(mixed, ref, 2.0, 4.0)
    elapsed = abs(d32.sum() / d64.sum() - 1.0)
    mu_bins = np.linspace(-1.0, 1.0, 17)
    p_bins = np.exp(np.linspace(np.log(0.04), np.log(4.0), 17))
    l1 = {}
    for key, bins in (("mu", mu_bins), ("p", p_bins)):
        h64 = np.histogram(ref[key], bins)[0]
        h32 = np.histogram(mixed[key], bins)[0]
        l1[key] = np.abs(h32 - h64).sum() / h64.sum()
    print("long", "focused" if focused else "parker", "dt", np.abs(d32 / d64 - 1).max(),
          "elapsed", elapsed, "l1", l1,
          {k: (float(np.quantile(v, 0.999)), float(v.max())) for k, v in dev.items()})
    if not focused:
        assert np.abs(d32 / d64 - 1.0).max() <= DT_REL
        assert np.array_equal(mixed["status"], ref["status"])
        assert np.quantile(dev["x"], 0.999) <= POS_REL
        assert np.quantile(dev["y"], 0.999) <= POS_REL
        assert np.quantile(dev["p"], 0.999) <= P_REL
    else:
        assert elapsed <= 0.01
        assert l1["mu"] <= 0.01 and l1["p"] <= 0.01
