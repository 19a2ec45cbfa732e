"""The header library's step API on the GPU against the reference's own code.

tests/golden/lib_*.npz were produced by the reference's ParkerSolver and
ParticleSystem templates (include/ParkerSolver.hpp, include/ParticleSystem.hpp)
compiled on the Kokkos-API shim, with the keyed Philox stream as the random
pool (tests/golden/make_golden.py).

* ParkerSolver: per-step dt within 1e-12 relative; positions, previous
  positions and momenta within the FP64 parity bar (1e-10 relative, periodic
  distance for wrapped coordinates); statuses and ids exact.  Both diffusion
  branches, periodic and open boundaries, stochastic and deterministic steps,
  and the graph-replayed multi-step call.
* FocusTransportSolver: the same bars, pitch cosines included (reflection at
  a maximum |mu| below 1, the three Picard iterations with the slab-QLT
  closure).
* Injected noise: both solvers stepped with caller normals (a tenth of
  them widened fourfold) against the reference templates fed the same
  normals through their random pool: the same bars.
* ParticleSystem: boundary conditions, sort_by_key, compact, energy split and
  capture_previous_positions bit for bit.
* Stored grids (lib_*_stored*.npz): the solver and lifecycle cases again on
  a StoredCoordinateGrid with stretched x and y faces (cell search by
  bisection, per-cell widths in the limiters): the same bars.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import lib_grid, load_golden

pytestmark = pytest.mark.gpu

FIELDS = ("x", "y", "prev_x", "prev_y", "prevstep_x", "prevstep_y", "p", "mu", "w", "e0",
          "status", "level", "key", "id")
PARKER_CASES = ("readme_periodic", "ratio_open", "readme_deterministic",
                "stored_readme_periodic", "stored_ratio_open", "stored_readme_deterministic")


def _state(data, prefix):
    return {k: data[f"{prefix}_{k}"].copy() for k in FIELDS}


def _compare(got, want, x_width, y_width, rtol=1e-10):
    for key in ("status", "level", "key", "id", "w", "mu", "e0"):
        assert np.array_equal(got[key], want[key]), key
    for key, width in (("x", x_width), ("prev_x", x_width), ("prevstep_x", x_width),
                       ("y", y_width), ("prev_y", y_width), ("prevstep_y", y_width)):
        diff = np.abs(got[key] - want[key])
        diff = np.minimum(diff, np.abs(width - diff)) / width
        assert diff.max() <= rtol, (key, diff.max())
    scale = np.maximum(np.abs(want["p"]), 1e-300)
    assert (np.abs(got["p"] - want["p"]) / scale).max() <= rtol


def _setup(ctx, data):
    grid = lib_grid(ctx, data)
    start = _state(data, "start")
    count = int(data["count"])
    system = ctx.system(count, start["x"].size)
    system.upload(start)
    solver = ctx.parker_solver(grid, data["basis"], bool(data["constant_ratio"]),
                               float(data["courant"]))
    return grid, system, solver


@pytest.mark.parametrize("case", PARKER_CASES)
def test_parker_solver_steps_match_reference(ctx, case):
    data = load_golden(f"lib_parker_{case}.npz")
    grid, system, solver = _setup(ctx, data)
    steps, first, seed = int(data["steps"]), int(data["first_step"]), int(data["seed"])
    dts = []
    for k in range(steps):
        if int(data["stochastic"]):
            dts.append(solver.advance_stochastic(system, seed, first + k))
        else:
            dts.append(solver.advance_deterministic(system))
    np.testing.assert_allclose(dts, data["dts"], rtol=1e-12, atol=0)
    got = system.download()
    want = _state(data, "end")
    width_x = data["x_edges"][-1] - data["x_edges"][0]
    width_y = data["y_edges"][-1] - data["y_edges"][0]
    _compare(got, want, width_x, width_y)
    assert system.count == int(data["count"])
    for h in (solver, system, grid):
        h.close()


def test_graph_replayed_steps_equal_single_steps(ctx):
    data = load_golden("lib_parker_readme_periodic.npz")
    grid, system, solver = _setup(ctx, data)
    steps, first, seed = int(data["steps"]), int(data["first_step"]), int(data["seed"])
    dts = solver.advance_stochastic_steps(system, seed, first, steps)
    np.testing.assert_allclose(dts, data["dts"], rtol=1e-12, atol=0)
    multi = system.download()
    grid2, system2, solver2 = _setup(ctx, data)
    for k in range(steps):
        solver2.advance_stochastic(system2, seed, first + k)
    single = system2.download()
    for key in FIELDS:
        assert np.array_equal(multi[key], single[key]), key
    for h in (solver, system, grid, solver2, system2, grid2):
        h.close()


def test_compute_time_step_is_the_first_step_dt(ctx):
    data = load_golden("lib_parker_readme_periodic.npz")
    grid, system, solver = _setup(ctx, data)
    assert solver.compute_time_step(system) == pytest.approx(float(data["dts"][0]), rel=1e-12)
    # compute_adaptive_time_step changes nothing
    before = _state(data, "start")
    after = system.download()
    for key in FIELDS:
        assert np.array_equal(after[key], before[key]), key
    solver.set_courant(0.6)
    assert solver.compute_time_step(system) == pytest.approx(2 * float(data["dts"][0]),
                                                             rel=1e-12)
    solver.set_courant(0.0)
    with pytest.raises(Exception, match="Courant"):
        solver.advance_stochastic(system, 1, 0)
    for h in (solver, system, grid):
        h.close()


def test_no_active_particle_is_an_error(ctx, kpt):
    data = load_golden("lib_parker_readme_periodic.npz")
    grid, system, solver = _setup(ctx, data)
    start = _state(data, "start")
    start["status"][:] = 2
    system.upload(start)
    assert solver.compute_time_step(system) == 0.0
    with pytest.raises(kpt.KptError, match="not positive and finite"):
        solver.advance_stochastic(system, 1, 0)
    for h in (solver, system, grid):
        h.close()


FOCUS_CASES = ("readme_periodic", "ratio_open_mumax", "deterministic",
               "stored_readme_periodic", "stored_ratio_open_mumax", "stored_deterministic")


def _focus_setup(ctx, data):
    grid = lib_grid(ctx, data)
    start = _state(data, "start")
    system = ctx.system(int(data["count"]), start["x"].size)
    system.upload(start)
    solver = ctx.focus_solver(grid, data["basis"], bool(data["constant_ratio"]),
                              float(data["courant"]), float(data["spectral_index"]),
                              float(data["h0"]), maximum_mu=float(data["max_mu"]))
    return grid, system, solver


@pytest.mark.parametrize("case", FOCUS_CASES)
def test_focus_solver_steps_match_reference(ctx, case):
    data = load_golden(f"lib_focus_{case}.npz")
    grid, system, solver = _focus_setup(ctx, data)
    steps, first, seed = int(data["steps"]), int(data["first_step"]), int(data["seed"])
    dts = []
    for k in range(steps):
        if int(data["stochastic"]):
            dts.append(solver.advance_stochastic(system, seed, first + k))
        else:
            dts.append(solver.advance_deterministic(system))
    # the pitch-angle limiters and reflections amplify last-bit pow/log
    # differences between the two builds to ~3e-12 in dt after one step
    np.testing.assert_allclose(dts, data["dts"], rtol=1e-10, atol=0)
    got = system.download()
    want = _state(data, "end")
    for key in ("status", "level", "key", "id", "w", "e0"):
        assert np.array_equal(got[key], want[key]), key
    width_x = data["x_edges"][-1] - data["x_edges"][0]
    width_y = data["y_edges"][-1] - data["y_edges"][0]
    for key, width in (("x", width_x), ("prev_x", width_x), ("prevstep_x", width_x),
                       ("y", width_y), ("prev_y", width_y), ("prevstep_y", width_y)):
        diff = np.abs(got[key] - want[key])
        diff = np.minimum(diff, np.abs(width - diff)) / width
        assert diff.max() <= 1e-10, (key, diff.max())
    for key in ("p", "mu"):
        scale = np.maximum(np.abs(want[key]), 1e-12)
        assert (np.abs(got[key] - want[key]) / scale).max() <= 1e-10, key
    for h in (solver, system, grid):
        h.close()


def test_focus_graph_steps_and_limits(ctx, kpt):
    data = load_golden("lib_focus_readme_periodic.npz")
    grid, system, solver = _focus_setup(ctx, data)
    assert solver.compute_time_step(system) == pytest.approx(float(data["dts"][0]), rel=1e-12)
    steps, first, seed = int(data["steps"]), int(data["first_step"]), int(data["seed"])
    dts = solver.advance_stochastic_steps(system, seed, first, steps)
    np.testing.assert_allclose(dts, data["dts"], rtol=1e-12, atol=0)
    with pytest.raises(kpt.KptError, match="maximum"):
        solver.set_maximum_mu(1.5)
    for h in (solver, system, grid):
        h.close()


@pytest.mark.parametrize("name", ["lib_system.npz", "lib_system_stored.npz"])
@pytest.mark.parametrize("op", ["boundary", "sort", "compact", "split", "capture"])
def test_particle_system_lifecycle_matches_reference(ctx, op, name):
    data = load_golden(name)
    grid = lib_grid(ctx, data)
    start = _state(data, "start")
    system = ctx.system(int(data["count"]), start["x"].size,
                        split_ratio=float(data["split_ratio"]),
                        min_child_weight=float(data["min_child_weight"]))
    system.upload(start)
    stats = None
    if op == "boundary":
        system.apply_boundary(grid)
    elif op == "sort":
        system.sort_by_key(-3, 40)
    elif op == "compact":
        system.compact()
    elif op == "split":
        stats = system.split_energy()
    else:
        system.capture_previous_positions()
    assert system.count == int(data[f"{op}_count"])
    want = _state(data, op)
    got = system.download()
    for key in FIELDS:
        assert np.array_equal(got[key], want[key]), key
    if stats is not None:
        assert [stats[k] for k in ("active_count", "split_count", "skipped_capacity_count",
                                   "skipped_invalid_baseline_count",
                                   "skipped_minimum_weight_count")] == \
            [int(v) for v in data["split_stats"]]
    system.close()
    grid.close()


@pytest.mark.parametrize("kind", ["parker", "focus"])
def test_injected_noise_steps_match_reference(ctx, kpt, kind):
    data = load_golden(f"lib_noise_{kind}.npz")
    if kind == "parker":
        grid, system, solver = _setup(ctx, data)
    else:
        grid, system, solver = _focus_setup(ctx, data)
    normals = data["normals"]
    with pytest.raises(kpt.KptError, match="normals must have shape"):
        solver.advance_with_noise(system, normals[0][:3])
    dts = [solver.advance_with_noise(system, normals[k]) for k in range(int(data["steps"]))]
    np.testing.assert_allclose(dts, data["dts"], rtol=1e-10, atol=0)
    got = system.download()
    want = _state(data, "end")
    for key in ("status", "level", "key", "id", "w", "e0"):
        assert np.array_equal(got[key], want[key]), key
    width_x = data["x_edges"][-1] - data["x_edges"][0]
    width_y = data["y_edges"][-1] - data["y_edges"][0]
    for key, width in (("x", width_x), ("prev_x", width_x), ("prevstep_x", width_x),
                       ("y", width_y), ("prev_y", width_y), ("prevstep_y", width_y)):
        diff = np.abs(got[key] - want[key])
        diff = np.minimum(diff, np.abs(width - diff)) / width
        assert diff.max() <= 1e-10, (key, diff.max())
    for key in ("p", "mu"):
        scale = np.maximum(np.abs(want[key]), 1e-12)
        assert (np.abs(got[key] - want[key]) / scale).max() <= 1e-10, key
    for h in (solver, system, grid):
        h.close()
