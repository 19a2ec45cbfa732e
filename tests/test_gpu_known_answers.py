"""Known-answer limits of the driver push, beside those of
test_gpu_statistics (uniform advection, adiabatic compression).

* Gradient drift: B = B_z(x) z with 1/B linear in x and no diffusion gives
  the Parker drift (src/main.cpp:1225-1236) v_y = vdp B_z' / B^2 = vdp c, a
  uniform drift along y, and no motion along x.
* Pitch-angle isotropisation: with a uniform field and no flow the focused
  push is pure pitch-angle diffusion; for the reduced closure with
  gamma_turb = 2 (D = duu0 (1 - mu^2)(|mu| + h0), whose derivative the
  driver writes consistently for that exponent, src/main.cpp:1551-1589) any
  start relaxes to the isotropic distribution, uniform over the clamp range
  [-mu_max, mu_max]: <mu> = 0, <mu^2> = mu_max^2 / 3.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_gradient_drift_is_uniform_along_y(ctx, kpt, fields_mod, binding):
    f = fields_mod.harris_field(256, 16, x_range=(0.0, 1.0), y_range=(0.0, 1.0))
    xc = 0.5 * (f.x_edges[1:] + f.x_edges[:-1])
    a, c = 2.0, 0.5
    bz = 1.0 / (a - c * xc)
    f.b[0], f.b[1] = 0.0, 0.0
    f.b[2] = np.broadcast_to(bz[None, :], f.b[2].shape).copy()
    f.v[0], f.v[1], f.v[2] = 0.0, 0.0, 0.0
    params = binding.default_params(kpara0=1e-30, kperp_over_kpara=0.0, dt_min_rel=1e-2,
                                    dt_max_rel=1e-2, drift_param1=1.0, drift_param2=0.0)
    settings = kpt.settings_from_dict(params)
    # vdp = 1 / (3 q) / sqrt((a1 p0 / p)^2 + (a2 p0^2 / p^2)^2) at p = p0
    vdy = 1.0 / (3.0 * params["charge"]) * c
    n = 2000
    rng = np.random.default_rng(4)
    arrays = binding.empty_particles(n)
    arrays.update(x=rng.uniform(0.3, 0.7, n), y=rng.uniform(0.0, 1.0, n),
                  p=np.full(n, params["p0"]), t=np.zeros(n), dt=np.full(n, 1e-3),
                  status=np.zeros(n, np.int32), w=np.ones(n))
    for precision, tol in ((kpt.PRECISION_F64, 1e-4), (kpt.PRECISION_MIXED, 1e-4)):
        lower = ctx.field(f, kpt.TABLE_PARKER16, precision)
        parts = ctx.particles(n)
        parts.upload(arrays, n)
        ctx.push_interval(parts, lower, lower, settings, 0, 17)
        got = parts.download()
        assert np.all(got["status"] == 0)
        dy = (got["y"] - arrays["y"] + 0.5) % 1.0 - 0.5
        want = vdy * params["mhd_dt"]
        assert np.abs(dy / want - 1.0).max() < tol, (precision, np.abs(dy / want - 1.0).max())
        assert np.abs(got["x"] - arrays["x"]).max() < 1e-9 * abs(want) + 1e-15, precision
        np.testing.assert_allclose(got["p"], arrays["p"], rtol=1e-14)
        for h in (parts, lower):
            h.close()


def test_pitch_angle_relaxes_to_isotropy(ctx, kpt, fields_mod, binding):
    f = fields_mod.harris_field(16, 16, x_range=(0.0, 1.0), y_range=(0.0, 1.0))
    f.b[0], f.b[1], f.b[2] = 1.0, 0.0, 0.0
    f.v[0], f.v[1], f.v[2] = 0.0, 0.0, 0.0
    # t = 10 relaxation times of the slowest mode; dt = 1e-3, small enough
    # that the clamped Euler-Maruyama step keeps the edge bins unbiased
    # (at dt = 1e-2 the reference's clamp piles ~10 % extra into them)
    params = binding.default_params(focused=1, closure=0, gamma_turb=2.0, duu0=1.0,
                                    kpara0=1e-30, kperp_over_kpara=0.0, mhd_dt=10.0,
                                    dt_min_rel=1e-4, dt_max_rel=1e-4)
    settings = kpt.settings_from_dict(params)
    n = 100000
    rng = np.random.default_rng(6)
    arrays = binding.empty_particles(n)
    arrays.update(x=rng.uniform(0.0, 1.0, n), y=rng.uniform(0.0, 1.0, n),
                  p=np.full(n, params["p0"]), t=np.zeros(n), dt=np.full(n, 1e-2),
                  mu=np.full(n, 0.7), status=np.zeros(n, np.int32), w=np.ones(n))
    mu_max = params["mu_max"]
    for precision in (kpt.PRECISION_F64, kpt.PRECISION_MIXED):
        lower = ctx.field(f, kpt.TABLE_FOCUSED21, precision)
        parts = ctx.particles(n)
        parts.upload(arrays, n)
        stats = ctx.push_interval(parts, lower, lower, settings, 0, 23)
        got = parts.download()
        assert stats.failed == 0 and np.all(got["status"] == 0)
        assert abs(stats.particle_steps / (n * 10000) - 1.0) < 2e-4
        mu = got["mu"]
        # the mixed push clamps at mu_max rounded to FP32
        assert np.abs(mu).max() <= max(mu_max, float(np.float32(mu_max)))
        # 100 000 samples: standard errors 0.0018 (<mu>) and 0.0009 (<mu^2>)
        assert abs(mu.mean()) < 0.008, (precision, mu.mean())
        assert abs((mu * mu).mean() - mu_max ** 2 / 3.0) < 0.005, (precision, (mu * mu).mean())
        hist = np.histogram(mu, bins=16, range=(-mu_max, mu_max))[0]
        assert np.abs(hist / hist.mean() - 1.0).max() < 0.08, (precision, hist)
        np.testing.assert_allclose(got["p"], arrays["p"], rtol=1e-14)
        for h in (parts, lower):
            h.close()
