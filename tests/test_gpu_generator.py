"""ParticleGenerator on the GPU against the reference's own templates.

tests/golden/lib_generator.npz was produced by include/ParticleGenerator.hpp
compiled on the Kokkos-API shim, its random pool drawing the keyed Philox
stream (tag 4, keyed by particle slot and frame); tests/golden/make_golden.py
made it.

* Every inject/recycle case ends bit for bit where the reference ends:
  positions (uniform draws, field-point coordinates and in-cell draws are
  formed with the same roundings), ids, statuses (accepted or inactive after
  the attempts run out), weights, kinetic-energy baselines, the particle
  count after commit_particle_range.
* Candidate sets: the compacted point indices exactly (stable, index order);
  cumulative physical-volume weights within 1e-13 relative (an FP64 scan
  associates its sums differently from the reference's serial scan).
* The reference's validation messages for empty candidate sets, bad plans,
  bad regions and out-of-range components.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import lib_grid, load_golden

pytestmark = pytest.mark.gpu

FIELDS = ("x", "y", "prev_x", "prev_y", "prevstep_x", "prevstep_y", "p", "mu", "w", "e0",
          "status", "level", "key", "id")


FILES = ("lib_generator.npz", "lib_generator_stored.npz")


@pytest.fixture(scope="module", params=FILES)
def gen(request):
    return load_golden(request.param)


def _setup(ctx, data):
    grid = lib_grid(ctx, data)
    fields = {}
    for name in ("scalar_cell", "vec_face", "mixed"):
        fields[name] = ctx.lib_field(grid, data[f"field_{name}"],
                                     tuple(int(c) for c in data[f"centering_{name}"]))
    return grid, fields


def _region(kpt, values):
    values = np.asarray(values, dtype=np.float64)
    if np.isnan(values).any():
        return None
    return kpt.make_particle_region(values[:2], values[2:])


def _run_case(kpt, ctx, grid, fields, data, name):
    case = data[f"{name}_case"]
    count, selection, seed, frame = int(case[1]), int(case[3]), int(case[4]), int(case[5])
    op = str(data[f"{name}_op"])
    field = fields[str(data[f"{name}_field"])]
    region = _region(kpt, data[f"{name}_region"])
    threshold, comparison, component, domain = data[f"{name}_predicate"]
    comparison, component, domain = int(comparison), int(component), int(domain)
    p, mu, weight, status = data[f"{name}_kinematics"]
    kin = kpt.ParticleInjectionKinematics(p, mu, weight, int(status))
    first, n, first_id, attempts = (int(v) for v in data[f"{name}_plan"])
    plan = kpt.ParticleInjectionPlan(first, n, first_id, attempts, 0)
    start = {k: data[f"{name}_start_{k}"] for k in FIELDS}
    system = ctx.system(count, start["x"].size)
    system.upload(start)
    rng = kpt.RandomManager(seed, frame)
    if op == "inject_uniform":
        kpt.inject_particles_uniform(system, rng, region, plan, kin)
    elif op == "inject_uniform_if":
        pred = kpt.make_field_threshold_particle_predicate(field, threshold, comparison,
                                                           component, domain)
        kpt.inject_particles_uniform_if(system, rng, region, plan, kin, pred)
    elif op == "inject_where_field":
        kpt.inject_particles_uniform_where_field(system, rng, plan, kin, field, threshold,
                                                 comparison, component, domain, region)
    elif op == "inject_in_grid":
        kpt.inject_particles_uniform_in_grid(system, rng, grid, plan, kin, domain)
    elif op == "recycle_uniform":
        kpt.recycle_particles_uniform(system, rng, region, kin, selection)
    elif op == "recycle_uniform_if":
        pred = kpt.make_field_threshold_particle_predicate(field, threshold, comparison,
                                                           component, domain)
        kpt.recycle_particles_uniform_if(system, rng, region, kin, pred, selection, attempts)
    elif op == "recycle_where_field":
        kpt.recycle_particles_uniform_where_field(system, rng, kin, field, threshold,
                                                  comparison, component, domain, selection,
                                                  region)
    elif op == "recycle_in_grid":
        kpt.recycle_particles_uniform_in_grid(system, rng, grid, kin, selection, domain)
    else:
        raise AssertionError(op)
    return system


@pytest.mark.parametrize("name", [str(c) for c in load_golden("lib_generator.npz")["cases"]])
def test_generator_matches_reference(ctx, kpt, gen, name):
    grid, fields = _setup(ctx, gen)
    system = _run_case(kpt, ctx, grid, fields, gen, name)
    assert system.count == int(gen[f"{name}_case"][2])
    got = system.download()
    for key in FIELDS:
        assert np.array_equal(got[key], gen[f"{name}_end_{key}"]), key
    for h in [system, grid] + list(fields.values()):
        h.close()


@pytest.mark.parametrize("name",
                         [str(c) for c in load_golden("lib_generator.npz")["candidate_cases"]])
def test_candidate_sets_match_reference(ctx, kpt, gen, name):
    grid, fields = _setup(ctx, gen)
    threshold, comparison, component, domain = gen[f"cand_{name}_predicate"]
    field = str(gen[f"cand_{name}_field"])
    if field:
        cands = ctx.make_field_particle_candidate_set(
            fields[field], threshold, int(comparison), int(component), int(domain),
            _region(kpt, gen[f"cand_{name}_region"]))
    else:
        cands = ctx.make_grid_particle_candidate_set(grid, int(domain))
    idx, cum = cands.download()
    want_idx = gen[f"cand_{name}_indices"]
    want_cum = gen[f"cand_{name}_cumulative"]
    assert cands.candidate_count() == want_idx.size
    assert np.array_equal(idx, want_idx)
    np.testing.assert_allclose(cum, want_cum, rtol=1e-13, atol=0)
    assert cands.total_weight() == pytest.approx(float(gen[f"cand_{name}_total"]), rel=1e-13)
    assert np.all(np.diff(cum) >= -1e-15 * cum[-1])
    for h in [cands, grid] + list(fields.values()):
        h.close()


def test_generator_errors_follow_the_reference(ctx, kpt, gen):
    grid, fields = _setup(ctx, gen)
    system = ctx.system(10, 64)
    rng = kpt.RandomManager(1, 0)
    kin = kpt.ParticleInjectionKinematics(1.0, 0.0, 1.0, 0)
    region = kpt.make_particle_region((-1.0, -1.0), (1.0, 1.0))
    with pytest.raises(kpt.KptError, match="first index is out of range"):
        kpt.inject_particles_uniform(system, rng, region,
                                     kpt.make_particle_injection_plan(11, 5), kin)
    with pytest.raises(kpt.KptError, match="requested range exceeds capacity"):
        kpt.inject_particles_uniform(system, rng, region,
                                     kpt.make_particle_injection_plan(10, 55), kin)
    with pytest.raises(kpt.KptError, match="max_attempts must be positive"):
        kpt.inject_particles_uniform(system, rng, region,
                                     kpt.make_particle_injection_plan(10, 5, 0), kin)
    with pytest.raises(kpt.KptError, match="weight must be positive"):
        kpt.inject_particles_uniform(system, rng, region,
                                     kpt.make_particle_injection_plan(10, 5),
                                     kpt.ParticleInjectionKinematics(1.0, 0.0, 0.0, 0))
    with pytest.raises(kpt.KptError, match="bounds must be finite and ascending"):
        kpt.make_particle_region((0.0, 0.0), (0.0, 1.0))
    with pytest.raises(kpt.KptError, match="component index is out of range"):
        ctx.make_field_particle_candidate_set(fields["scalar_cell"], 0.0, "greater", 1)
    with pytest.raises(kpt.KptError, match="no candidate grid points"):
        kpt.inject_particles_uniform_where_field(system, rng,
                                                 kpt.make_particle_append_plan(system, 5), kin,
                                                 fields["scalar_cell"], 1e9, "greater")
    with pytest.raises(kpt.KptError, match="recycling has no candidate grid points"):
        kpt.recycle_particles_uniform_where_field(system, rng, kin, fields["scalar_cell"], 1e9,
                                                  "greater")
    assert system.count == 10
    # an append plan commits its range: the count grows to first index + count
    kpt.inject_particles_uniform(system, rng, region, kpt.make_particle_append_plan(system, 7),
                                 kin)
    assert system.count == 17
    got = system.download()
    assert np.array_equal(got["id"][10:17], np.arange(10, 17, dtype=np.uint64))
    assert np.all(got["status"][10:17] == 0)
    for h in [system, grid] + list(fields.values()):
        h.close()


def test_recycling_is_schedule_independent(ctx, kpt, gen):
    """Each particle slot draws from its own stream: recycling the same
    population twice, or the same slots inside a larger population, gives
    the same particles."""
    grid, fields = _setup(ctx, gen)
    rng = kpt.RandomManager(99, 5)
    kin = kpt.ParticleInjectionKinematics(0.5, 0.1, 1.0, 0)
    n = 3000
    start = {k: gen[f"recycle_in_grid_start_{k}"] for k in FIELDS}
    base = {k: np.resize(v, n) for k, v in start.items()}
    base["id"] = np.arange(n, dtype=np.uint64)
    runs = []
    for count in (n, n // 3):
        system = ctx.system(count, n)
        system.upload(base)
        kpt.recycle_particles_uniform_in_grid(system, rng, grid, kin, "recyclable")
        runs.append(system.download())
        system.close()
    for key in FIELDS:
        assert np.array_equal(runs[0][key][: n // 3], runs[1][key][: n // 3]), key
    for h in [grid] + list(fields.values()):
        h.close()
