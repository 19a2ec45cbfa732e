"""The C-ABI library loads on the CPU and exports every symbol kpt.h declares."""
from __future__ import annotations

import ctypes
import os
import subprocess

import pytest


def test_library_exports_every_declared_function(kpt):
    path = kpt.library_path()
    if not os.path.exists(path):
        import __graft_entry__
        __graft_entry__.build_library()
    lib = ctypes.CDLL(path)
    declared = kpt.header_functions()
    assert len(declared) >= 20
    missing = [name for name in declared if not hasattr(lib, name)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True,
                         check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T kpt_" in line}
    assert set(declared) <= exported


def test_no_device_fails_loudly(kpt):
    """Without a GPU the context cannot be created: there is no CPU path."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(kpt.KptError):
        kpt.Context(0)


def test_abi_version_and_defaults(kpt):
    lib = kpt.load_library()
    assert lib.kpt_abi_version() == 2
    s = kpt.default_settings()
    assert s.mhd_dt == 0.1 and s.p0 == 0.1 and s.max_steps == 200000
    assert s.kperp_over_kpara == 0.01 and s.split_ratio == 2.0
