"""Momentum and pitch-cosine spectra of a particle population, and how two
spectra are compared.

Binning follows the driver's momentum histogram (src/main.cpp:1907-1964):
log bins of [pmin, pmax], ``bin = int((ln p - ln pmin) * nbins / ln(pmax /
pmin))`` clamped to the range, the weights of active particles (status 0)
with pmin <= p <= pmax summed per bin.  The comparison follows the
reference's accuracy script (scripts/run_local_parker_focused_speed_accuracy_test.sh:105-121):
relative L1 = sum |c - r| / sum |r| and the largest per-bin relative
difference.  Beside it, a two-sample chi-square test of the two histograms
(the reference has none) says whether they are consistent within Monte Carlo
error.

Two kinds of comparison are meaningful for a stochastic push:

* **paired** -- both runs draw the same keyed noise (same seed), so the
  particles follow nearly the same paths and the histograms differ only by
  the arithmetic (precision, closure).  The L1 measures that systematic
  difference directly; a chi-square test between paired runs is
  conservative (correlated samples agree better than independent ones).
* **independent** -- the candidate draws other noise (another seed) from the
  same start; the chi-square test then is a real Monte Carlo test of the
  two distributions, while the L1 carries the Monte Carlo noise of both.

Weights enter the chi-square test as counts.  That is exact for unit
weights (no splitting) and an approximation for dyadic split weights.
"""
from __future__ import annotations

from typing import Dict, Optional, Sequence

import numpy as np


def momentum_spectrum(p, w, status, nbins: int = 64, pmin: float = 1e-2,
                      pmax: float = 1e1) -> np.ndarray:
    """Weight per log-momentum bin of the active particles (the driver's
    binning, src/main.cpp:1913-1941)."""
    p, w, status = np.asarray(p), np.asarray(w), np.asarray(status)
    active = (status == 0) & (p >= pmin) & (p <= pmax)
    bins = np.floor((np.log(p[active]) - np.log(pmin)) * nbins / np.log(pmax / pmin))
    bins = np.clip(bins.astype(np.int64), 0, nbins - 1)
    return np.bincount(bins, weights=w[active], minlength=nbins).astype(np.float64)


def pitch_spectrum(mu, w, status, nbins: int = 16) -> np.ndarray:
    """Weight per pitch-cosine bin of [-1, 1] of the active particles."""
    mu, w, status = np.asarray(mu), np.asarray(w), np.asarray(status)
    active = status == 0
    return np.histogram(mu[active], bins=nbins, range=(-1.0, 1.0),
                        weights=w[active])[0].astype(np.float64)


def fine_log_momentum_edges(p, status, p0: float, nbins: int = 64,
                            tail: float = 0.005) -> np.ndarray:
    """Edges of a fine ln(p/p0) histogram fitted to a reference population:
    `nbins` equal bins between its `tail` and 1 - `tail` quantiles, and one
    open bin on either side (so no particle is lost)."""
    lnp = np.log(np.asarray(p)[np.asarray(status) == 0] / p0)
    lo, hi = np.quantile(lnp, [tail, 1.0 - tail])
    if not hi > lo:
        hi = lo + 1e-12
    inner = np.linspace(lo, hi, nbins + 1)
    return np.concatenate(([-np.inf], inner, [np.inf]))


def log_momentum_histogram(p, w, status, p0: float, edges: np.ndarray) -> np.ndarray:
    """Weight per ln(p/p0) bin (edges from fine_log_momentum_edges)."""
    p, w, status = np.asarray(p), np.asarray(w), np.asarray(status)
    active = status == 0
    return np.histogram(np.log(p[active] / p0), bins=edges,
                        weights=w[active])[0].astype(np.float64)


def relative_l1(candidate: np.ndarray, reference: np.ndarray):
    """(sum |c - r| / sum |r|, max_i |c_i - r_i| / max(|r_i|, 1e-12 max |r|)),
    the two figures of the reference's accuracy script."""
    c = np.asarray(candidate, dtype=np.float64)
    r = np.asarray(reference, dtype=np.float64)
    denom = np.abs(r).sum()
    diff = np.abs(c - r)
    l1 = float(diff.sum() / denom) if denom > 0 else float("nan")
    floor = np.abs(r).max() * 1e-12 if np.any(r != 0) else 1.0
    max_rel = float(np.max(diff / np.maximum(np.abs(r), floor))) if r.size else float("nan")
    return l1, max_rel


def chi2_two_sample(a: np.ndarray, b: np.ndarray, min_count: float = 10.0) -> Dict[str, float]:
    """Two-sample chi-square test of histograms a and b (totals may differ):
    chi2 = sum_i (sqrt(B/A) a_i - sqrt(A/B) b_i)^2 / (a_i + b_i) over the bins
    with a_i + b_i >= min_count, the remaining bins pooled into one more
    bin; dof = bins used - 1.  Returns chi2, dof and the p-value (1.0 when
    fewer than two bins are populated)."""
    from scipy import stats as sps
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    total = a + b
    keep = total >= min_count
    aa, bb = list(a[keep]), list(b[keep])
    rest_a, rest_b = a[~keep].sum(), b[~keep].sum()
    if rest_a + rest_b > 0:
        aa.append(rest_a)
        bb.append(rest_b)
    aa, bb = np.array(aa), np.array(bb)
    A, B = aa.sum(), bb.sum()
    if len(aa) < 2 or A <= 0 or B <= 0:
        return {"chi2": 0.0, "dof": 0, "p_value": 1.0}
    chi2 = float(np.sum((np.sqrt(B / A) * aa - np.sqrt(A / B) * bb) ** 2 / (aa + bb)))
    dof = len(aa) - 1
    return {"chi2": chi2, "dof": int(dof), "p_value": float(sps.chi2.sf(chi2, dof))}


def compare(candidate: np.ndarray, reference: np.ndarray) -> Dict[str, float]:
    """Relative L1, largest per-bin relative difference, and the chi-square
    test of a candidate histogram against a reference one."""
    l1, max_rel = relative_l1(candidate, reference)
    out = {"l1": l1, "max_rel": max_rel,
           "populated_bins": int(np.count_nonzero(np.asarray(reference)))}
    out.update(chi2_two_sample(candidate, reference))
    return out


def population_spectra(state: Dict[str, np.ndarray], p0: float,
                       fine_edges: Optional[np.ndarray] = None) -> Dict[str, np.ndarray]:
    """The three histograms a comparison uses: 64 driver bins of p, a fine
    ln(p/p0) histogram (edges given, usually fitted to the reference) and 16
    pitch-cosine bins."""
    out = {"p64": momentum_spectrum(state["p"], state["w"], state["status"])}
    if fine_edges is not None:
        out["lnp_fine"] = log_momentum_histogram(state["p"], state["w"], state["status"], p0,
                                                 fine_edges)
    if "mu" in state:
        out["mu16"] = pitch_spectrum(state["mu"], state["w"], state["status"])
    return out


def compare_populations(candidate: Dict[str, np.ndarray], reference: Dict[str, np.ndarray],
                        p0: float, keys: Sequence[str] = ("p64", "lnp_fine", "mu16")
                        ) -> Dict[str, Dict[str, float]]:
    """compare() on each histogram of two particle populations, the fine
    ln(p/p0) edges fitted to the reference."""
    edges = fine_log_momentum_edges(reference["p"], reference["status"], p0)
    ref = population_spectra(reference, p0, edges)
    got = population_spectra(candidate, p0, edges)
    out = {key: compare(got[key], ref[key]) for key in keys if key in ref and key in got}
    out["bins_with_1pct_weight"] = int(np.count_nonzero(ref["p64"] >= 0.01 * ref["p64"].sum()))
    return out
