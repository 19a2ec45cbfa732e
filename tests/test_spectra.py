"""The spectrum comparison behind the metric's accuracy bar, on the CPU.

* The histograms follow the driver's binning (src/main.cpp:1913-1941) and
  the relative L1 the reference's accuracy script
  (scripts/run_local_parker_focused_speed_accuracy_test.sh:105-121).
* The two-sample chi-square test accepts two samples of one distribution and
  rejects samples of different ones.
* The bar has teeth: on oracle runs of the focused push with the slab-QLT
  closure, a planted closure error (sigma^2 1.5 times too large) fails the
  paired 1 % pitch-cosine L1, and a planted 1 % momentum bias fails the
  chi-square test of the fine ln(p/p0) histogram, while the unchanged
  oracle passes both.
"""
from __future__ import annotations

import importlib

import numpy as np
import pytest

spectra = importlib.import_module("kokkos-particletransport_gb300.spectra")


def test_momentum_spectrum_uses_the_driver_binning():
    rng = np.random.default_rng(1)
    p = np.exp(rng.uniform(np.log(5e-3), np.log(2e1), 5000))
    w = 0.5 ** rng.integers(0, 4, p.size)
    status = rng.choice([0, 0, 0, 1, 2], p.size).astype(np.int32)
    got = spectra.momentum_spectrum(p, w, status, nbins=128)
    want = np.zeros(128)
    lmin, scale = np.log(1e-2), 128 / np.log(1e3)
    for pk, wk, sk in zip(p, w, status):
        if sk == 0 and 1e-2 <= pk <= 1e1:
            want[min(max(int((np.log(pk) - lmin) * scale), 0), 127)] += wk
    np.testing.assert_array_equal(got, want)


def test_relative_l1_is_the_reference_scripts_figure():
    r = np.array([4.0, 2.0, 0.0, 2.0])
    c = np.array([3.0, 2.0, 1.0, 2.0])
    l1, max_rel = spectra.relative_l1(c, r)
    assert l1 == pytest.approx(2.0 / 8.0)
    assert max_rel == pytest.approx(1.0 / (4.0 * 1e-12))  # the empty bin's floor


def test_chi_square_accepts_one_distribution_and_rejects_two():
    rng = np.random.default_rng(2)
    probs = np.exp(-0.5 * ((np.arange(40) - 20) / 5.0) ** 2)
    probs /= probs.sum()
    a = rng.multinomial(200000, probs).astype(float)
    b = rng.multinomial(150000, probs).astype(float)
    same = spectra.chi2_two_sample(a, b)
    assert same["p_value"] > 0.01 and same["dof"] >= 20
    shifted = np.roll(probs, 1)  # the mean moved by a fifth of the width
    c = rng.multinomial(150000, shifted / shifted.sum()).astype(float)
    assert spectra.chi2_two_sample(a, c)["p_value"] < 1e-6
    assert spectra.chi2_two_sample(a, a)["p_value"] == 1.0


N, INTERVALS, SUBSTEPS, FRAME, SEED = 8192, 5, 200, 7, 99


def _params(binding, **changes):
    rel = (1.0 + 1e-6) / SUBSTEPS
    values = dict(kperp_over_kpara=0.05, focused=1, closure=1, qlt_sigma2=0.1,
                  qlt_spectral_index=5.0 / 3.0, dt_min_rel=rel, dt_max_rel=rel)
    values.update(changes)
    return binding.default_params(**values)


@pytest.fixture(scope="module")
def oracle_runs(binding, oracle, fields_mod):
    ye = fields_mod.stretched_edges(128, -2.0, 2.0, strength=4.0)
    f0 = fields_mod.harris_field(64, 128, y_edges=ye, island_amplitude=0.1, noise=0.01, seed=5)
    f1 = fields_mod.harris_field(64, 128, y_edges=ye, island_amplitude=0.1, noise=0.01, seed=6)
    grid = oracle.grid(f0.x_edges, f0.y_edges)
    lo, up = oracle.table(f0, True), oracle.table(f1, True)
    start = binding.empty_particles(N)
    oracle.inject(grid, _params(binding), FRAME * 0.1, FRAME, SEED, N, 0, N, start)
    start["status"][:] = 0
    start["t"][:] = FRAME * 0.1

    def run(params, seed):
        state = {k: v.copy() for k, v in start.items()}
        for k in range(INTERVALS):
            oracle.push(grid, lo, up, params, (FRAME + k) * 0.1, FRAME + k, seed, N, state)
        return state

    runs = {"ref": run(_params(binding), SEED),
            "same_seed": run(_params(binding), SEED),
            "other_seed": run(_params(binding), SEED + 1),
            "closure_error": run(_params(binding, qlt_sigma2=0.15), SEED)}
    oracle.free_grid(grid)
    return runs


def test_unchanged_oracle_passes_the_bar(oracle_runs):
    ref = oracle_runs["ref"]
    same = spectra.compare_populations(oracle_runs["same_seed"], ref, 0.1)
    assert all(same[k]["l1"] == 0.0 for k in ("p64", "lnp_fine", "mu16"))
    other = spectra.compare_populations(oracle_runs["other_seed"], ref, 0.1)
    assert all(other[k]["p_value"] > 0.01 for k in ("p64", "lnp_fine", "mu16"))


def test_planted_closure_error_fails_the_paired_l1(oracle_runs):
    got = spectra.compare_populations(oracle_runs["closure_error"], oracle_runs["ref"], 0.1)
    assert got["mu16"]["l1"] > 0.01, got["mu16"]


def test_planted_momentum_bias_fails_the_chi_square(oracle_runs):
    biased = dict(oracle_runs["other_seed"])
    biased["p"] = biased["p"] * 1.01
    got = spectra.compare_populations(biased, oracle_runs["ref"], 0.1)
    assert got["lnp_fine"]["p_value"] <= 0.01, got["lnp_fine"]
