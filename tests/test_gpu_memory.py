"""Calls that allocate device scratch give it back: repeating them does not
shrink the free device memory (the candidate sets, the coefficient
precompute, the surrogate's evaluation and gradient, the library solvers)."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _free_bytes(ctx):
    import torch
    ctx.synchronize()
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


def test_repeated_calls_do_not_leak_device_memory(ctx, kpt, fields_mod, binding):
    nx, ny = 512, 512
    xe = np.linspace(-1.0, 1.0, nx + 1)
    ye = np.linspace(-2.0, 2.0, ny + 1)
    grid = ctx.grid(xe, ye, (1, 0))
    points = (nx + 4) * (ny + 4)
    rng = np.random.default_rng(3)
    b = np.stack([1.0 + 0.1 * rng.standard_normal(points), 0.1 * rng.standard_normal(points),
                  0.3 + 0.0 * rng.standard_normal(points)], axis=1)
    v = 0.1 * rng.standard_normal((points, 3))
    field = ctx.lib_field(grid, rng.standard_normal(points))
    params = binding.default_params(kperp_over_kpara=0.05, focused=1, closure=2)
    surrogate = ctx.train_surrogate(kpt.settings_from_dict(params), samples=65536, steps=50,
                                    batch=4096)
    _, norm = surrogate.parameters()
    inputs = np.column_stack([np.full(50000, 0.5), np.full(50000, np.log(params["p0"])),
                              np.zeros(50000), np.full(50000, 0.1), np.full(50000, 5.0 / 3.0)])
    x = rng.uniform(-1, 1, (20000, 5)).astype(np.float32)
    t = rng.normal(0, 1, (20000, 3)).astype(np.float32)
    weights = np.zeros(surrogate.parameter_count, dtype=np.float32)

    def round_of_calls():
        cands = ctx.make_field_particle_candidate_set(field, 0.0, "greater")
        cands.close()
        cands = ctx.make_grid_particle_candidate_set(grid)
        cands.close()
        ctx.parker_coefficients(grid, b, v)
        ctx.focus_coefficients(grid, b, v)
        surrogate.evaluate(inputs)
        ctx.surrogate_gradient(weights, x, t, surrogate.hidden_width)

    round_of_calls()  # first-use allocations (context buffers, module loading)
    before = _free_bytes(ctx)
    for _ in range(10):
        round_of_calls()
    after = _free_bytes(ctx)
    # one round holds ~60 MB of scratch; a leak of it would cost 600 MB here
    assert before - after < 32 * 1024 * 1024, (before - after) / 2**20
    ctx.set_surrogate(None)
    surrogate.close()
    field.close()
    grid.close()


def test_download_into_caller_arrays(ctx, kpt, fields_mod, binding):
    """ParticleStorage.download(out=...) fills caller arrays (the bench's
    pinned buffers) with what a plain download returns, and refuses arrays
    of the wrong type or length."""
    f = fields_mod.harris_field(32, 64, noise=0.01, seed=1)
    settings = kpt.settings_from_dict(binding.default_params(kperp_over_kpara=0.05))
    lower = ctx.field(f)
    parts = ctx.particles(1000)
    ctx.inject(parts, lower, settings, 700, 3, 11)
    want = parts.download()
    out = {k: np.full(1000, 7, dtype=v.dtype) for k, v in want.items()}
    got = parts.download(out=out)
    assert got is out
    for k in want:
        assert np.array_equal(out[k][:want[k].size], want[k]), k
        assert np.all(out[k][want[k].size:] == 7), k
    bad = dict(out, p=np.zeros(1000, dtype=np.float32))
    with pytest.raises(kpt.KptError, match="contiguous"):
        parts.download(out=bad)
    short = dict(out, x=np.zeros(10))
    with pytest.raises(kpt.KptError, match="length"):
        parts.download(out=short)
    for h in (parts, lower):
        h.close()
