"""The headline workload's step rule, on the oracle (no GPU): with the step
fixed at (1 + 1e-6) mhd_dt / N every particle takes exactly N steps per
interval (the last one cut to the interval end), where mhd_dt / N itself
leaves a rounding remainder for one more, tiny step."""
from __future__ import annotations

import importlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _steps(oracle, binding, fields_mod, dt_rel, n=64, intervals=2):
    f0 = fields_mod.harris_field(32, 64, noise=0.01, seed=1)
    f1 = fields_mod.harris_field(32, 64, noise=0.01, seed=2)
    params = binding.default_params(kperp_over_kpara=0.05, focused=1, closure=1,
                                    dt_min_rel=dt_rel, dt_max_rel=dt_rel)
    grid = oracle.grid(f0.x_edges, f0.y_edges)
    parts = binding.empty_particles(n)
    frame = 100
    oracle.inject(grid, params, frame * params["mhd_dt"], frame, 7, n, 0, n, parts)
    parts["status"][:] = 0
    parts["t"][:] = frame * params["mhd_dt"]
    counts = []
    for k in range(intervals):
        counts.append(oracle.push(grid, oracle.table(f0, True), oracle.table(f1, True), params,
                                  (frame + k) * params["mhd_dt"], frame + k, 7, n, parts))
    oracle.free_grid(grid)
    return np.concatenate(counts)


def test_fixed_step_rule_gives_exactly_n_steps(oracle, binding, fields_mod):
    sys.path.insert(0, ROOT)
    bench = importlib.import_module("bench")

    class _Kpt:  # the two attributes fixed_step_settings reads
        CLOSURE_QLT = 1

        @staticmethod
        def default_settings(**kw):
            return type("S", (), dict(kw, dt_min_rel=0.0, dt_max_rel=0.0))()

    for n in (100, 1000):
        settings = bench.fixed_step_settings(_Kpt, 1, n)
        assert settings.dt_min_rel == settings.dt_max_rel == (1.0 + 1e-6) / n
        counts = _steps(oracle, binding, fields_mod, settings.dt_min_rel)
        assert np.all(counts == n), (n, np.unique(counts))
    # the plain 1/N step can leave a remainder for one more step
    assert np.all(_steps(oracle, binding, fields_mod, 1.0 / 1000) == 1001)


def test_tensor_flop_model_and_engine_choice():
    """The bench's tensor-rate model (flops per network evaluation as each
    engine issues them) and the engine a network of each width starts on."""
    sys.path.insert(0, ROOT)
    bench = importlib.import_module("bench")
    assert bench.tensor_flop_per_step(64, "tcgen05") == 14848
    assert bench.tensor_flop_per_step(32, "tcgen05") == 5632
    assert bench.tensor_flop_per_step(32, "mma.sync") == 3584
    assert bench.default_engine(64) == "tcgen05"
    assert bench.default_engine(32) == "mma.sync"
    assert set(bench.PROFILES_HEAD) == {"tcgen05", "mma.sync"}
    for engine, path in bench.PROFILES_HEAD.items():
        for key in ("dram_bytes_per_particle_step", "l1tex_data_pipe_frac",
                    "issue_active_frac"):
            assert bench.profile_value(path, key) is not None, (engine, key)
