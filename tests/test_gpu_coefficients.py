"""Coefficient precompute on the GPU against the reference's own code.

tests/golden/lib_parker_coefficients.npz holds the packed basis the
reference's ParkerSolver builds from make_legacy_transport_coefficient_fields
(include/ParkerCoefficient.hpp:1102-1155) for four configurations (README and
constant-ratio branches, constant and per-point turbulence, floors, both
ghost-fill modes, open and periodic axes), compiled on the Kokkos-API shim
(tests/golden/make_golden.py).

* B, V, curl(B/B^2) and div V use only correctly rounded operations in the
  reference's order: bit for bit, ghost cells included.
* The gamma-one kappas go through pow, whose last bits differ between the
  CUDA and host math libraries: 1e-14 relative.
* The diffusion-tensor divergence bases are three-point differences of those
  kappas: 1e-12 of each component's largest magnitude.
* The reference's abort messages for a magnetic null and a negative Lc.
* lib_*_coefficients_stored.npz: the same configurations on a
  StoredCoordinateGrid with stretched faces (three-point differences on the
  stored coordinates): the same bars.

tests/golden/lib_focus_coefficients.npz does the same for the focused
builder (include/FocusCoefficient.hpp:852-993) and the focused packed basis:
B, b, V, |B|, the curvature drift basis, div V, bb:grad V, b.dV/dt, sigma^2
and Lc bit for bit; the kappas 1e-14; ln|B|-derived entries (gradient drift
basis, focusing) and the perpendicular diffusion advection 1e-12 of scale
(log and pow differ in their last bits between the two math libraries).
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import lib_grid, load_golden

pytestmark = pytest.mark.gpu

# the uniform (analytic) grid's files and the stored (explicit, stretched
# faces) grid's files hold the same configurations
PARKER_FILES = ("lib_parker_coefficients.npz", "lib_parker_coefficients_stored.npz")
FOCUS_FILES = ("lib_focus_coefficients.npz", "lib_focus_coefficients_stored.npz")
_LOADED = {}


def _golden(name):
    if name not in _LOADED:
        _LOADED[name] = load_golden(name)
    return _LOADED[name]


CASES = [(f, str(c)) for f in PARKER_FILES for c in _golden(f)["cases"]]
FOCUS_CASES = [(f, str(c)) for f in FOCUS_FILES for c in _golden(f)["cases"]]


@pytest.fixture(scope="module")
def coef():
    return _golden("lib_parker_coefficients.npz")


def _inputs(ctx, data, name):
    grid = lib_grid(ctx, data, data[f"{name}_periodic"])
    s2, l2d, lslab, lc = data[f"{name}_turbulence"]
    fields = data[f"{name}_fields"]
    if fields.size:
        turbulence = {"sigma2_field": fields[0], "l2d_field": fields[1],
                      "lslab_field": fields[2], "lc_field": fields[3]}
    else:
        turbulence = {"sigma2": s2, "l2d": l2d, "lslab": lslab, "lc": lc}
    (model, pf, pp, ratio, min_b, min_vsw, min_sigma2, floor, ghost,
     charge) = data[f"{name}_params"]
    params = ctx.diffusion_parameters(
        perpendicular_model=int(model), ghost_fill_mode=int(ghost), parallel_prefactor=pf,
        perpendicular_prefactor=pp, perpendicular_parallel_ratio=ratio,
        minimum_magnetic_field_magnitude=min_b, minimum_solar_wind_speed=min_vsw,
        minimum_sigma2=min_sigma2, minimum_magnetic_field_squared_for_drift=floor)
    return grid, turbulence, params, float(charge)


@pytest.mark.parametrize("file,name", CASES)
def test_packed_basis_matches_reference(ctx, file, name):
    coef = _golden(file)
    grid, turbulence, params, charge = _inputs(ctx, coef, name)
    got = ctx.parker_coefficients(grid, coef[f"{name}_b"], coef[f"{name}_v"], turbulence,
                                  params, charge=charge)
    want = coef[f"{name}_packed"]
    exact = list(range(0, 9)) + [17]
    assert np.array_equal(got[:, exact], want[:, exact])
    np.testing.assert_allclose(got[:, 15:17], want[:, 15:17], rtol=1e-14, atol=0)
    for c in range(9, 15):
        scale = max(np.abs(want[:, c]).max(), 1e-300)
        assert np.abs(got[:, c] - want[:, c]).max() <= 1e-12 * scale, c
    grid.close()


def test_solver_from_fields_equals_solver_from_basis(ctx, kpt, coef):
    """The basis built on the device drives the same steps as the same
    basis uploaded from the host."""
    name = "readme_constant"
    grid, turbulence, params, charge = _inputs(ctx, coef, name)
    b, v = coef[f"{name}_b"], coef[f"{name}_v"]
    basis = ctx.parker_coefficients(grid, b, v, turbulence, params, charge=charge)
    rng = np.random.default_rng(5)
    n = 2000
    state = {"id": np.arange(n, dtype=np.uint64)}
    for key in kpt.SYSTEM_DOUBLE_FIELDS:
        state[key] = np.zeros(n)
    for key in kpt.SYSTEM_INT_FIELDS:
        state[key] = np.zeros(n, dtype=np.int32)
    xe, ye = coef["x_edges"], coef["y_edges"]
    state["x"] = rng.uniform(xe[0], xe[-1], n)
    state["y"] = rng.uniform(ye[0] + 0.5, ye[-1] - 0.5, n)
    state["p"] = np.exp(rng.uniform(np.log(0.05), np.log(3.0), n))
    state["w"] = np.ones(n)
    results = []
    for solver in (ctx.parker_solver_from_fields(grid, b, v, turbulence, params, charge=charge),
                   ctx.parker_solver(grid, basis)):
        system = ctx.system(n, n, charge=charge)
        system.upload(state)
        dts = solver.advance_stochastic_steps(system, 9, 0, 3)
        results.append((dts, system.download()))
        solver.close()
        system.close()
    assert np.array_equal(results[0][0], results[1][0])
    for key in ("x", "y", "p", "status"):
        assert np.array_equal(results[0][1][key], results[1][1][key]), key
    grid.close()


def test_failures_report_the_reference_messages(ctx, kpt, coef):
    grid = ctx.grid(coef["x_edges"], coef["y_edges"], (1, 0))
    messages = dict(zip([str(n) for n in coef["error_names"]],
                        [str(m) for m in coef["error_messages"]]))
    with pytest.raises(kpt.KptError) as info:
        ctx.parker_coefficients(grid, coef["error_zero_b"], coef["error_v"])
    assert messages["zero_b"] in str(info.value)
    lc_fields = coef["error_negative_lc"]
    turbulence = {"sigma2_field": lc_fields[0], "l2d_field": lc_fields[1],
                  "lslab_field": lc_fields[2], "lc_field": lc_fields[3]}
    with pytest.raises(kpt.KptError) as info:
        ctx.parker_coefficients(grid, coef["error_b"], coef["error_v"], turbulence)
    assert messages["negative_lc"] in str(info.value)
    with pytest.raises(kpt.KptError, match="constant perpendicular ratio must be positive"):
        ctx.parker_coefficients(grid, coef["error_b"], coef["error_v"],
                                parameters=ctx.diffusion_parameters(perpendicular_model=1))
    grid.close()


@pytest.fixture(scope="module")
def fcoef():
    return _golden("lib_focus_coefficients.npz")


def _focus_inputs(ctx, data, name):
    grid, turbulence, params, charge = _inputs(ctx, data, name)
    dvdt = data[f"{name}_dvdt"]
    floor = float(data[f"{name}_params"][7])
    return grid, turbulence, params, charge, (dvdt if dvdt.size else None), floor


@pytest.mark.parametrize("file,name", FOCUS_CASES)
def test_focus_packed_basis_matches_reference(ctx, file, name):
    fcoef = _golden(file)
    grid, turbulence, params, charge, dvdt, floor = _focus_inputs(ctx, fcoef, name)
    # the Parker floor slot carries the builder's floor for the focused cases
    params.minimum_magnetic_field_squared_for_drift = 0.0
    got = ctx.focus_coefficients(grid, fcoef[f"{name}_b"], fcoef[f"{name}_v"], dvdt, turbulence,
                                 params, floor, charge=charge)
    want = fcoef[f"{name}_packed"]
    exact = list(range(0, 9)) + [12, 13, 14, 18, 21, 23, 24, 25, 26]
    for c in exact:
        assert np.array_equal(got[:, c], want[:, c]), c
    np.testing.assert_allclose(got[:, 19:21], want[:, 19:21], rtol=1e-14, atol=0)
    for c in (9, 10, 11, 15, 16, 17, 22):
        scale = max(np.abs(want[:, c]).max(), 1e-300)
        assert np.abs(got[:, c] - want[:, c]).max() <= 1e-12 * scale, c
    grid.close()


def test_focus_solver_from_fields_equals_solver_from_basis(ctx, kpt, fcoef):
    name = "ratio_floors_dvdt"
    grid, turbulence, params, charge, dvdt, floor = _focus_inputs(ctx, fcoef, name)
    params.minimum_magnetic_field_squared_for_drift = 0.0
    b, v = fcoef[f"{name}_b"], fcoef[f"{name}_v"]
    basis = ctx.focus_coefficients(grid, b, v, dvdt, turbulence, params, floor, charge=charge)
    rng = np.random.default_rng(6)
    n = 1500
    state = {"id": np.arange(n, dtype=np.uint64)}
    for key in kpt.SYSTEM_DOUBLE_FIELDS:
        state[key] = np.zeros(n)
    for key in kpt.SYSTEM_INT_FIELDS:
        state[key] = np.zeros(n, dtype=np.int32)
    xe, ye = fcoef["x_edges"], fcoef["y_edges"]
    state["x"] = rng.uniform(xe[0], xe[-1], n)
    state["y"] = rng.uniform(ye[0] + 0.5, ye[-1] - 0.5, n)
    state["p"] = np.exp(rng.uniform(np.log(0.05), np.log(3.0), n))
    state["mu"] = rng.uniform(-1.0, 1.0, n)
    state["w"] = np.ones(n)
    results = []
    ratio = params.perpendicular_model == 1
    for solver in (ctx.focus_solver_from_fields(grid, b, v, dvdt, turbulence, params, floor,
                                                charge=charge),
                   ctx.focus_solver(grid, basis, ratio)):
        system = ctx.system(n, n, charge=charge)
        system.upload(state)
        dts = solver.advance_stochastic_steps(system, 4, 0, 3)
        results.append((dts, system.download()))
        solver.close()
        system.close()
    assert np.array_equal(results[0][0], results[1][0])
    for key in ("x", "y", "p", "mu", "status"):
        assert np.array_equal(results[0][1][key], results[1][1][key]), key
    grid.close()


def test_focus_direction_of_a_null_field_fails_like_the_reference(ctx, kpt, coef):
    grid = ctx.grid(coef["x_edges"], coef["y_edges"], (1, 0))
    with pytest.raises(kpt.KptError, match="direction is undefined at zero magnitude"):
        ctx.focus_coefficients(grid, coef["error_zero_b"], coef["error_v"])
    grid.close()
