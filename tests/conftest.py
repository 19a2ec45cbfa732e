"""Shared fixtures.  GPU tests carry @pytest.mark.gpu; everything else runs on CPU."""
from __future__ import annotations

import importlib
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
for path in (ROOT, os.path.join(ROOT, "oracle")):
    if path not in sys.path:
        sys.path.insert(0, path)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libkpt.so")


@pytest.fixture(scope="session")
def kpt():
    return importlib.import_module("kokkos-particletransport_gb300")


@pytest.fixture(scope="session")
def fields_mod():
    return importlib.import_module("kokkos-particletransport_gb300.fields")


@pytest.fixture(scope="session")
def binding():
    return importlib.import_module("binding")


@pytest.fixture(scope="session")
def oracle(binding):
    return binding.Oracle()


@pytest.fixture(scope="session")
def ctx(kpt):
    with kpt.Context(0) as context:
        yield context


def load_golden(name: str) -> dict:
    with np.load(os.path.join(GOLDEN, name), allow_pickle=False) as data:
        return {k: data[k] for k in data.files}


def lib_grid(ctx, data: dict, periodic=None):
    """The library grid of a golden file: a stored grid on its x_faces /
    y_faces when it has them, else the analytic grid on its uniform edges."""
    periodic = data["periodic"] if periodic is None else periodic
    if "x_faces" in data:
        return ctx.stored_grid(data["x_faces"], data["y_faces"], periodic)
    return ctx.grid(data["x_edges"], data["y_edges"], periodic)


def golden_params(data: dict) -> dict:
    """A fixture's parameters over the oracle defaults (closure fields included)."""
    binding = importlib.import_module("binding")
    out = binding.default_params()
    for n, v in zip([str(n) for n in data["param_names"]], data["param_values"]):
        out[n] = int(v) if isinstance(out.get(n), int) else float(v)
    return out


def golden_field(data: dict, prefix: str):
    fields = importlib.import_module("kokkos-particletransport_gb300.fields")
    return fields.CompactField(data[f"{prefix}_x_edges"], data[f"{prefix}_y_edges"],
                               data[f"{prefix}_b"], data[f"{prefix}_v"])


def golden_particles(data: dict, prefix: str) -> dict:
    names = ("x", "y", "p", "t", "dt", "w", "mu", "status", "level")
    return {n: data[f"{prefix}_{n}"].copy() for n in names}
