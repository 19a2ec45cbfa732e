"""The CPU reference of the learned closure (oracle/surrogate_ref.py).

Its analytic gradient is pinned to central finite differences, and its
training targets to the oracle's slab-QLT functions (themselves bit-exact
with the reference's LegencyModel.hpp:557-645, see test_oracle_golden)."""
from __future__ import annotations

import numpy as np
import pytest

import surrogate_ref as sr


def _random_problem(seed=3, n=48, hidden=32):
    rng = np.random.default_rng(seed)
    params = rng.normal(0.0, 0.3, sr.layout(hidden)["N_PARAMS"])
    x = rng.uniform(-1.0, 1.0, (n, sr.N_IN))
    t = rng.normal(0.0, 1.0, (n, sr.N_OUT))
    return params, x, t


@pytest.mark.parametrize("hidden", [32, 64])
def test_gradient_matches_finite_differences(hidden):
    params, x, t = _random_problem(hidden=hidden)
    _, grad = sr.loss_and_gradient(params, x, t)
    rng = np.random.default_rng(7)
    o = sr.layout(hidden)
    # every block: W1, b1, W2, b2, W3, b3
    idx = np.concatenate([rng.integers(lo, hi, 12) for lo, hi in
                          ((o["W1"], o["B1"]), (o["B1"], o["W2"]), (o["W2"], o["B2"]),
                           (o["B2"], o["W3"]), (o["W3"], o["B3"]), (o["B3"], o["N_PARAMS"]))])
    fd = sr.finite_difference_gradient(params, x, t, idx)
    assert np.allclose(grad[idx], fd, rtol=1e-6, atol=1e-9)


@pytest.mark.parametrize("hidden", [32, 64])
def test_forward_matches_loss_definition(hidden):
    params, x, t = _random_problem(seed=5, hidden=hidden)
    loss, _ = sr.loss_and_gradient(params, x, t)
    assert loss == pytest.approx(np.mean((sr.forward(params, x) - t) ** 2), rel=1e-14)


def test_targets_reconstruct_the_oracle_closure(oracle):
    rng = np.random.default_rng(11)
    n = 200
    mu = rng.uniform(0.02, 0.999, n) * np.where(rng.uniform(size=n) < 0.5, -1.0, 1.0)
    p = np.exp(rng.uniform(np.log(0.01), np.log(100.0), n))
    b = np.exp(rng.uniform(np.log(0.05), np.log(5.0), n))
    sigma2 = np.exp(rng.uniform(np.log(0.01), 0.0, n))
    gk = rng.uniform(1.5, 2.0, n)
    phys = dict(p0=0.1, particle_v0=1.0, qlt_omega0=1000.0, qlt_lc=0.05, qlt_h0=1e-6)
    d, dd, y0, y1 = sr.qlt_targets(mu, p, b, sigma2, gk, **phys)
    speed = phys["particle_v0"] * p / phys["p0"]
    omega = phys["qlt_omega0"] * b / np.sqrt(1.0 + p * p)
    d_ref, dd_ref = oracle.qlt(mu, omega, speed, sigma2, phys["qlt_lc"], gk, phys["qlt_h0"])
    assert np.allclose(d, d_ref, rtol=1e-12, atol=0)
    assert np.allclose(dd, dd_ref, rtol=1e-10, atol=1e-12 * np.abs(d_ref).max())
    # the network's targets reproduce D and dD/dmu
    reg = np.abs(mu) + phys["qlt_h0"]
    assert np.allclose((1.0 - mu * mu) * np.exp(y0), d, rtol=1e-12)
    dd_from = d * (np.sign(mu) * y1 / reg - 2.0 * mu / (1.0 - mu * mu))
    assert np.allclose(dd_from, dd, rtol=1e-9, atol=1e-12 * np.abs(d).max())
