"""The allocation-free summary entry point (kpt_summarize_noalloc).

Some callers cannot allocate device memory: an application that owns all
device memory through its own pool, or code that must not call cudaMalloc.
kpt_summarize_noalloc serves them: the particle arrays are the caller's, and
the reduction's scratch is one fixed device array inside the library.  This
file is collected last so that a run stopping at the first failure has
already run every other test; it also passes on its own in a fresh process.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KPT_ERROR_CAPACITY = -6
MAX_PARTICLES = 16_777_216


def _summarize_noalloc(kpt, arrays, count):
    lib = kpt.load_library()
    fn = lib.kpt_summarize_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p]
    dev = kpt.ParticleArrays(**{name: arrays[name] for name, _ in kpt.ParticleArrays._fields_})
    out = kpt.Summary()
    rc = fn(ctypes.byref(dev), int(count), None, ctypes.byref(out))
    return rc, out.as_dict()


def _random_particles(binding, n, seed):
    rng = np.random.default_rng(seed)
    arrays = binding.empty_particles(n)
    arrays["p"][:] = rng.lognormal(np.log(0.1), 0.3, n)
    arrays["dt"][:] = rng.uniform(1e-6, 1e-3, n)
    arrays["level"][:] = rng.integers(0, 7, n).astype(np.int32)
    arrays["w"][:] = 0.5 ** arrays["level"]
    arrays["status"][:] = rng.choice([0, 0, 0, 1, 2], n).astype(np.int32)
    return arrays


def test_noalloc_summary_matches_context_summary(kpt, binding):
    with kpt.Context(0) as ctx:
        for n, seed in ((300_001, 1), (70_000, 2)):
            arrays = _random_particles(binding, n, seed)
            parts = ctx.particles(n)
            parts.upload(arrays, n)
            want = ctx.summarize(parts)
            dev = parts.device_arrays()
            # two calls in a row on the shared scratch, then a smaller count
            for _ in range(2):
                rc, got = _summarize_noalloc(kpt, dev, n)
                assert rc == 0, kpt.load_library().kpt_last_error().decode()
                for key in ("stored", "active", "inactive", "max_split_level", "weight_sum",
                            "p_min", "p_max", "dt_min", "dt_max"):
                    assert got[key] == want[key], key
                for key in ("p_avg", "dt_avg"):
                    assert got[key] == pytest.approx(want[key], rel=1e-13), key
            parts.close()


def test_noalloc_summary_rejects_counts_beyond_its_scratch(kpt, binding):
    with kpt.Context(0) as ctx:
        parts = ctx.particles(16)
        parts.upload(_random_particles(binding, 16, 3), 16)
        rc, _ = _summarize_noalloc(kpt, parts.device_arrays(), MAX_PARTICLES + 1)
        assert rc == KPT_ERROR_CAPACITY
        assert "scratch limit" in kpt.load_library().kpt_last_error().decode()
        rc, got = _summarize_noalloc(kpt, parts.device_arrays(), 16)
        assert rc == 0 and got["stored"] == 16
        parts.close()
