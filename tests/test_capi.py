"""CPU checks of the C ABI library: it builds for sm_103a, loads, and
exports every function include/mgpu_gb300.h declares.  No compute calls."""
import ctypes
import os

import pytest


def test_library_exports_declared_symbols(mgpu):
    from mgpu_gb300 import _lib
    names = _lib.declared_functions()
    assert len(names) >= 20
    handle = ctypes.CDLL(_lib.library_path())
    missing = [n for n in names if not hasattr(handle, n)]
    assert not missing, missing


def test_status_strings(mgpu):
    lib = mgpu.lib()
    for code in range(8):
        assert lib.mgpu_status_string(code)


def test_null_context_rejected(mgpu):
    lib = mgpu.lib()
    assert lib.mgpu_synchronize(None) == 1
    assert lib.mgpu_radix_sort(None, 1, None, 0, None, 0, None, None) == 1


def test_no_cpu_fallback_symbols(mgpu):
    """The product library does not link the oracle."""
    from mgpu_gb300 import _lib
    handle = ctypes.CDLL(_lib.library_path())
    for name in ("oracle_sort", "emu_radix_sort", "oracle_merge"):
        assert not hasattr(handle, name)
