"""The project pow (kokkos-particletransport_gb300/csrc/kpt_pow.h) on the CPU.

The FP64 push, the C restatement and the reference build on the shim all
compute x^y with it, so the GPU and the host round every power alike.  Here
it is pinned on the host: accuracy against 200-bit evaluations (below 0.52
ulp on the argument ranges the push uses and across the double range), the
host C library's pow (equal in all but a few tenths of a percent of cases,
never more than one ulp apart), C99 Annex F special values, and the
constants in the header (ln 2 split, series coefficients) recomputed here.
The GPU evaluation of the same function is compared bit for bit in
tests/test_gpu_parity.py.
"""
from __future__ import annotations

import ctypes
import os
import re

import numpy as np
import pytest

mp = pytest.importorskip("mpmath")

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                      "kokkos-particletransport_gb300", "csrc", "kpt_pow.h")


def _libm_pow():
    libm = ctypes.CDLL("libm.so.6")
    libm.pow.restype = ctypes.c_double
    libm.pow.argtypes = [ctypes.c_double, ctypes.c_double]
    return libm.pow


def _cases(n=1500):
    rng = np.random.default_rng(11)
    return [
        ("wide", np.exp(rng.uniform(-8, 8, n)), rng.uniform(-3, 3, n)),
        ("|mu|^(gamma-1)", rng.uniform(0, 1, n), np.full(n, 5 / 3 - 1)),
        ("|mu|^(gamma-2)", rng.uniform(1e-6, 1, n), np.full(n, 5 / 3 - 2)),
        ("B^(gamma-2)", np.exp(rng.uniform(-3, 3, n)), np.full(n, 1.6666667 - 2)),
        ("(p/p0)^(3-gamma)", np.exp(rng.uniform(-5, 8, n)), np.full(n, 3 - 1.6666667)),
        ("near 1", 1 + rng.uniform(-1e-3, 1e-3, n), rng.uniform(-50, 50, n)),
        ("full range", np.exp(rng.uniform(-700, 700, n)), rng.uniform(-1, 1, n)),
        ("split ladder", np.full(64, 1.2), np.arange(64, dtype=float)),
    ]


@pytest.mark.parametrize("name,x,y", _cases())
def test_pow_is_within_052_ulp_and_agrees_with_libm(oracle, name, x, y):
    mp.mp.prec = 200
    got = oracle.pow(x, y)
    libm_pow = _libm_pow()
    ref = np.array([libm_pow(float(a), float(b)) for a, b in zip(x, y)])
    worst = 0.0
    for xi, yi, g in zip(x, y, got):
        exact = mp.power(mp.mpf(float(xi)), mp.mpf(float(yi)))
        worst = max(worst, float(abs(mp.mpf(float(g)) - exact) / np.spacing(abs(g))))
    assert worst < 0.52, worst
    differ = got != ref
    assert differ.sum() <= max(1, 0.01 * differ.size), differ.mean()
    assert np.all(np.abs(got[differ] - ref[differ]) <= np.spacing(np.abs(ref[differ]))), name


def test_pow_special_values_follow_c99(oracle):
    libm_pow = _libm_pow()
    values = [0.0, -0.0, 1.0, -1.0, 2.0, -2.0, 0.5, -0.5, 3.0, -3.0, np.inf, -np.inf, np.nan,
              1e-310, -1e-310, 1e308, 0.1, -1e-7]
    for a in values:
        for b in values:
            got = oracle.pow([a], [b])[0]
            want = libm_pow(a, b)
            if np.isnan(want):
                assert np.isnan(got), (a, b)
            else:
                assert got == want and np.signbit(got) == np.signbit(want), (a, b, got, want)


def test_pow_constants_are_the_stated_values():
    text = open(HEADER).read()
    mp.mp.prec = 200

    def hexval(comment):
        m = re.search(r"(0x[0-9a-f.]+p[-+]\d+)\)?;\s*/\* " + re.escape(comment) + r" \*/", text)
        assert m, comment
        return float.fromhex(m.group(1))

    for k in range(1, 13):
        assert hexval(f"2/{2 * k + 1}") == float(mp.mpf(2) / (2 * k + 1)), k
    for n in range(3, 16):
        assert hexval(f"1/{n}!") == float(1 / mp.factorial(n)), n
    hi = float.fromhex(re.search(r"LN2_HI = (0x[0-9a-f.]+p[-+]\d+);", text).group(1))
    lo = float.fromhex(re.search(r"LN2_LO = (0x[0-9a-f.]+p[-+]\d+);", text).group(1))
    mant = mp.mpf(hi) * 2 ** 42  # hi in [1/2, 1) with 42 significant bits
    assert mant == int(mant) and 2 ** 41 <= mant < 2 ** 42
    assert lo == float(mp.log(2) - mp.mpf(hi))
