"""Comparison helpers with the tolerances the parity tests use."""
from __future__ import annotations

import numpy as np

# FP64 GPU vs oracle: trajectories within 1e-10 relative.  Positions are
# compared modulo the periodic width and relative to it; momentum, time and
# step size relative to their own magnitude.
F64_REL = 1.0e-10


def periodic_diff(a, b, width):
    d = np.asarray(a) - np.asarray(b)
    return np.abs(d - width * np.round(d / width))


def rel_diff(a, b, floor=1e-300):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.abs(a - b) / np.maximum(np.abs(b), floor)


def trajectory_errors(got: dict, want: dict, x_width: float, y_width: float,
                      focused: bool) -> dict:
    errs = {
        "x": float(np.max(periodic_diff(got["x"], want["x"], x_width) / x_width, initial=0.0)),
        "y": float(np.max(periodic_diff(got["y"], want["y"], y_width) / y_width, initial=0.0)),
        "p": float(np.max(rel_diff(got["p"], want["p"]), initial=0.0)),
        "t": float(np.max(rel_diff(got["t"], want["t"]), initial=0.0)),
        "dt": float(np.max(rel_diff(got["dt"], want["dt"]), initial=0.0)),
    }
    if focused:
        errs["mu"] = float(np.max(np.abs(np.asarray(got["mu"]) - want["mu"]), initial=0.0))
    return errs
