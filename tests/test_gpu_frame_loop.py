"""The driver's frame loop on the C2-type field (stretched y edges, Harris
sheet plus islands, a freshly noised frame per interval), at a reduced size:
every interval injects, pushes and splits (split ratio 1.2), every fourth
frame bins the momentum histogram -- on the GPU in FP64 and through the
oracle.  The reference's reader rejects stretched edges, so the oracle's
restatement is the reference here.

* FP64: particle count, ids (order included), statuses and split levels bit
  for bit; positions and momenta within the 1e-10 parity bar; every
  histogram identical -- in storage order and in the CLI's tile order.
* Mixed precision: the final momentum spectrum within 1 % L1 of the
  oracle's, chi-square p > 0.01.
* Focused transport with the slab-QLT closure through the same loop (the
  pitch-angle dynamics amplify last-bit differences over an interval, so
  FP64 is held to the statistical bar here, as mixed precision is): the
  same particle counts, momentum spectra within 1 % L1 and chi-square
  p > 0.01, pitch-cosine distributions chi-square p > 0.01.
"""
from __future__ import annotations

import numpy as np
import pytest

from test_gpu_statistics import _chi2_same, _spectrum

pytestmark = pytest.mark.gpu

FRAMES, REQUESTED, CAPACITY, SEED = 8, 900, 16384, 2024  # FRAMES intervals


def _frames(fields_mod):
    ye = fields_mod.stretched_edges(256, -2.0, 2.0)
    return [fields_mod.harris_field(128, 256, y_edges=ye, island_amplitude=0.1, noise=0.01,
                                    seed=100 + f) for f in range(FRAMES + 1)]


def _oracle_loop(oracle, binding, params, frames):
    grid = oracle.grid(frames[0].x_edges, frames[0].y_edges)
    tables = [oracle.table(f, bool(params["focused"])) for f in frames]
    ref = binding.empty_particles(CAPACITY)
    count, hists, splits = 0, [], []
    for f in range(len(frames) - 1):
        count = oracle.inject(grid, params, f * params["mhd_dt"], f, SEED, CAPACITY, count,
                              REQUESTED, ref, band=(-0.2, 0.2))
        oracle.push(grid, tables[f], tables[f + 1], params, f * params["mhd_dt"], f, SEED,
                    count, ref)
        count, split, skipped = oracle.split(params, CAPACITY, count, ref)
        splits.append((split, skipped))
        if (f + 1) % 4 == 0:
            hists.append(oracle.histogram(params["pmin"], params["pmax"], 128, count, ref))
    oracle.free_grid(grid)
    return {k: v[:count] for k, v in ref.items()}, hists, splits


def _gpu_loop(ctx, kpt, params, frames, precision, order=None):
    settings = kpt.settings_from_dict(params)
    kind = kpt.TABLE_FOCUSED21 if params["focused"] else kpt.TABLE_PARKER16
    fields = [ctx.field(f, kind, precision) for f in frames]
    parts = ctx.particles(CAPACITY)
    hists, splits = [], []
    for f in range(len(frames) - 1):
        ctx.inject(parts, fields[f], settings, REQUESTED, f, SEED, band=(-0.2, 0.2))
        if order == "tiles":
            ctx.sort(parts, fields[f], 8, 8)
        ctx.push_interval(parts, fields[f], fields[f + 1], settings, f, SEED)
        splits.append(ctx.split(parts, settings))
        if (f + 1) % 4 == 0:
            hists.append(ctx.histogram(parts, params["pmin"], params["pmax"], 128))
    got = parts.download()
    for h in fields + [parts]:
        h.close()
    return got, hists, splits


@pytest.fixture(scope="module")
def loop_reference(oracle, binding, fields_mod):
    params = binding.default_params(kperp_over_kpara=0.05, split_ratio=1.2)
    frames = _frames(fields_mod)
    return params, frames, _oracle_loop(oracle, binding, params, frames)


@pytest.mark.parametrize("order", [None, "tiles"])
def test_frame_loop_f64_matches_oracle(ctx, kpt, loop_reference, order):
    """The work order (storage order, or the CLI's tile order) changes nothing."""
    params, frames, (ref, ref_hists, ref_splits) = loop_reference
    got, hists, splits = _gpu_loop(ctx, kpt, params, frames, kpt.PRECISION_F64, order)
    assert sum(s for s, _ in ref_splits) > 0  # the ladder is exercised
    assert splits == ref_splits
    assert got["x"].size == ref["x"].size
    for key in ("status", "level"):
        assert np.array_equal(got[key], ref[key]), key
    np.testing.assert_array_equal(got["w"], ref["w"])
    for key, width in (("x", 2.0), ("y", 4.0)):
        d = np.abs(got[key] - ref[key])
        d = np.minimum(d, width - d) / width
        assert d.max() <= 1e-10, (key, d.max())
    assert (np.abs(got["p"] - ref["p"]) / ref["p"]).max() <= 1e-10
    for h, h_ref in zip(hists, ref_hists):
        assert np.array_equal(h, h_ref)


def test_frame_loop_mixed_spectrum(ctx, kpt, loop_reference):
    params, frames, (ref, _, _) = loop_reference
    got, _, _ = _gpu_loop(ctx, kpt, params, frames, kpt.PRECISION_MIXED)
    h_ref = _spectrum(ref["p"], ref["w"], ref["status"])
    h = _spectrum(got["p"], got["w"], got["status"])
    assert np.abs(h - h_ref).sum() / h_ref.sum() <= 0.01
    assert _chi2_same(h, h_ref) > 0.01


def test_focused_qlt_frame_loop_statistics(ctx, kpt, oracle, binding, fields_mod):
    params = binding.default_params(kperp_over_kpara=0.05, split_ratio=1.2, focused=1,
                                    closure=1)
    frames = _frames(fields_mod)[:5]  # 4 intervals
    ref, _, ref_splits = _oracle_loop(oracle, binding, params, frames)
    h_ref = _spectrum(ref["p"], ref["w"], ref["status"])
    mu_ref = np.histogram(ref["mu"][ref["status"] == 0], bins=16, range=(-1, 1))[0]
    for precision in (kpt.PRECISION_F64, kpt.PRECISION_MIXED):
        got, _, splits = _gpu_loop(ctx, kpt, params, frames, precision)
        # injected particles: the count less the children
        assert got["x"].size - sum(s for s, _ in splits) == \
            ref["x"].size - sum(s for s, _ in ref_splits)
        h = _spectrum(got["p"], got["w"], got["status"])
        assert np.abs(h - h_ref).sum() / h_ref.sum() <= 0.01, precision
        assert _chi2_same(h, h_ref) > 0.01, precision
        mu = np.histogram(got["mu"][got["status"] == 0], bins=16, range=(-1, 1))[0]
        assert _chi2_same(mu.astype(float), mu_ref.astype(float)) > 0.01, precision
