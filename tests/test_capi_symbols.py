"""The C-ABI library loads without a GPU and exports every entry point that
include/ccake_gpu.h declares (no compute calls are made here)."""
import ctypes
import os
import subprocess

import pytest

from ccake_gb300 import api, build


def _lib_or_skip():
    try:
        build.build()
    except RuntimeError as e:  # no nvcc in this environment
        pytest.skip(str(e))
    return build.LIB


def test_library_exports_every_declared_symbol():
    path = _lib_or_skip()
    L = ctypes.CDLL(path)
    names = api.exported_symbols()
    assert len(names) >= 18
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_status_strings_without_gpu():
    L = api.lib()
    assert L.ccake_status_string(0) == b"ok"
    assert L.ccake_status_string(3) == b"EoS inversion failed"


def test_no_cpu_fallback_symbols():
    # the product library must not contain the oracle
    path = _lib_or_skip()
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True).stdout
    assert "orc_" not in out
