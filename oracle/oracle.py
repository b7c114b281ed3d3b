"""ctypes access to the host oracle (test infrastructure, not product code).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module.  It loads oracle/lib/liboracle_mgpu.so (built by oracle/build.py
from oracle.cpp and ref_emulation.cpp) and wraps its functions for numpy
arrays.
"""
import ctypes
import os

import numpy as np

from . import build as _build

DTYPE_CODES = {
    np.dtype(np.int32): 0,
    np.dtype(np.uint32): 1,
    np.dtype(np.float32): 2,
    np.dtype(np.int64): 3,
    np.dtype(np.uint64): 4,
    np.dtype(np.float64): 5,
}
OPS = {"plus": 0, "max": 1, "min": 2}
MODES = {"less": 0, "greater": 1, "radix": 2}

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        _lib = ctypes.CDLL(path)
        vp, i64, i32, dbl = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_double
        sig = {
            "oracle_sort": [i32, vp, i32, vp, i64, i32],
            "oracle_sort_parallel": [i32, vp, i32, vp, i64, i32, i32],
            "oracle_merge": [i32, vp, vp, i64, vp, vp, i64, vp, vp, i32, i32],
            "oracle_scan_int": [i32, vp, vp, i64, i32, vp, i32],
            "oracle_scan_fp": [i32, vp, vp, vp, i64, i32, dbl, i32],
            "oracle_segmented_sort": [i32, vp, i32, vp, vp, i64, i32],
            "oracle_segmented_scan_int": [i32, vp, vp, vp, i64, i32, vp, i32],
            "oracle_to_radix_bits": [i32, vp, vp, i64],
            "oracle_scan_int_parallel": [i32, vp, vp, i64, i32, i32],
            "emu_mergesort": [i32, vp, vp, i32, i32, i32, i32, i32, i32],
            "emu_merge": [i32, vp, vp, i32, vp, vp, i32, vp, vp, i32, i32, i32, i32],
            "emu_scan_exc_i32": [vp, i32, i32, i32, ctypes.c_int32],
            "emu_radix_sort": [i32, vp, vp, i32, i32, i32, i32],
            "emu_libc_rand_fill": [vp, i64, ctypes.c_uint],
        }
        for name, args in sig.items():
            f = getattr(_lib, name)
            f.argtypes = args
            f.restype = None if name == "emu_libc_rand_fill" else i32
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _vb(vals):
    return 0 if vals is None else vals.dtype.itemsize


def _check(rc):
    if rc != 0:
        raise ValueError("oracle call rejected its arguments (rc=%d)" % rc)


def sort(keys, vals=None, mode="less"):
    """Stable sort (std::stable_sort) of copies of keys/vals; returns them."""
    k = np.ascontiguousarray(keys).copy()
    v = None if vals is None else np.ascontiguousarray(vals).copy()
    _check(lib().oracle_sort(DTYPE_CODES[k.dtype], _ptr(k), _vb(v), _ptr(v), k.size, MODES[mode]))
    return k, v


def sort_parallel(keys, vals=None, mode="less", threads=None):
    k = np.ascontiguousarray(keys).copy()
    v = None if vals is None else np.ascontiguousarray(vals).copy()
    threads = threads or os.cpu_count() or 1
    _check(lib().oracle_sort_parallel(DTYPE_CODES[k.dtype], _ptr(k), _vb(v), _ptr(v), k.size,
                                      MODES[mode], threads))
    return k, v


def sort_parallel_inplace(keys, vals, mode, threads):
    """Same as sort_parallel but sorts the given arrays in place (for timing)."""
    _check(lib().oracle_sort_parallel(DTYPE_CODES[keys.dtype], _ptr(keys), _vb(vals), _ptr(vals),
                                      keys.size, MODES[mode], threads))


def radix_sort(keys, vals=None):
    """Stable sort by radix bits (the radix_sort order)."""
    return sort(keys, vals, mode="radix")


def merge(a_keys, a_vals, b_keys, b_vals, mode="less"):
    a_keys = np.ascontiguousarray(a_keys)
    b_keys = np.ascontiguousarray(b_keys)
    c_keys = np.empty(a_keys.size + b_keys.size, a_keys.dtype)
    c_vals = None
    if a_vals is not None:
        a_vals = np.ascontiguousarray(a_vals)
        b_vals = np.ascontiguousarray(b_vals)
        c_vals = np.empty(c_keys.size, a_vals.dtype)
    _check(lib().oracle_merge(DTYPE_CODES[a_keys.dtype], _ptr(a_keys), _ptr(a_vals), a_keys.size,
                              _ptr(b_keys), _ptr(b_vals), b_keys.size, _ptr(c_keys), _ptr(c_vals),
                              _vb(a_vals), MODES[mode]))
    return c_keys, c_vals


def scan_int(x, exclusive=True, init=0, op="plus"):
    x = np.ascontiguousarray(x)
    out = np.empty_like(x)
    init_a = np.array([init], dtype=x.dtype)
    _check(lib().oracle_scan_int(DTYPE_CODES[x.dtype], _ptr(x), _ptr(out), x.size, int(exclusive),
                                 _ptr(init_a), OPS[op]))
    return out


def scan_fp(x, exclusive=False, init=0.0, op="plus"):
    """Float scan accumulated in double.  Returns (scan, prefix of |x|)."""
    x = np.ascontiguousarray(x)
    out = np.empty(x.size, np.float64)
    out_abs = np.empty(x.size, np.float64)
    _check(lib().oracle_scan_fp(DTYPE_CODES[x.dtype], _ptr(x), _ptr(out), _ptr(out_abs), x.size,
                                int(exclusive), float(init), OPS[op]))
    return out, out_abs


def segmented_sort(keys, vals, offsets, mode="radix"):
    k = np.ascontiguousarray(keys).copy()
    v = None if vals is None else np.ascontiguousarray(vals).copy()
    off = np.ascontiguousarray(offsets, dtype=np.int64)
    _check(lib().oracle_segmented_sort(DTYPE_CODES[k.dtype], _ptr(k), _vb(v), _ptr(v), _ptr(off),
                                       off.size - 1, MODES[mode]))
    return k, v


def segmented_scan_int(x, offsets, exclusive=False, init=0, op="plus"):
    x = np.ascontiguousarray(x)
    out = np.empty_like(x)
    off = np.ascontiguousarray(offsets, dtype=np.int64)
    init_a = np.array([init], dtype=x.dtype)
    _check(lib().oracle_segmented_scan_int(DTYPE_CODES[x.dtype], _ptr(x), _ptr(out), _ptr(off),
                                           off.size - 1, int(exclusive), _ptr(init_a), OPS[op]))
    return out


def to_radix_bits(keys):
    keys = np.ascontiguousarray(keys)
    out = np.empty(keys.size, np.uint32 if keys.dtype.itemsize == 4 else np.uint64)
    _check(lib().oracle_to_radix_bits(DTYPE_CODES[keys.dtype], _ptr(keys), _ptr(out), keys.size))
    return out


def scan_int_parallel_inplace(x, out, exclusive, threads):
    _check(lib().oracle_scan_int_parallel(DTYPE_CODES[x.dtype], _ptr(x), _ptr(out), x.size,
                                          int(exclusive), threads))


# --- restatement of the reference's tile algorithms (ref_emulation.cpp) ---

EMU_KEYS = {np.dtype(np.int32): 0, np.dtype(np.uint32): 1, np.dtype(np.float32): 2,
            np.dtype(np.uint64): 4}


def emu_mergesort(keys, vals=None, nt=128, vt=7, sort_indices=False, comp="less"):
    k = np.ascontiguousarray(keys).copy()
    v = None
    if vals is not None or sort_indices:
        v = np.zeros(k.size, np.int32) if vals is None else np.ascontiguousarray(vals, np.int32).copy()
    _check(lib().emu_mergesort(EMU_KEYS[k.dtype], _ptr(k), _ptr(v), k.size, nt, vt,
                               int(vals is not None), int(sort_indices), MODES[comp]))
    return k, v


def emu_merge(a_keys, a_vals, b_keys, b_vals, nt=128, vt=7, comp="less"):
    a_keys = np.ascontiguousarray(a_keys)
    b_keys = np.ascontiguousarray(b_keys)
    c_keys = np.empty(a_keys.size + b_keys.size, a_keys.dtype)
    c_vals = None
    if a_vals is not None:
        a_vals = np.ascontiguousarray(a_vals, np.int32)
        b_vals = np.ascontiguousarray(b_vals, np.int32)
        c_vals = np.empty(c_keys.size, np.int32)
    _check(lib().emu_merge(EMU_KEYS[a_keys.dtype], _ptr(a_keys), _ptr(a_vals), a_keys.size,
                           _ptr(b_keys), _ptr(b_vals), b_keys.size, _ptr(c_keys), _ptr(c_vals),
                           nt, vt, int(a_vals is not None), MODES[comp]))
    return c_keys, c_vals


def emu_scan_exc_i32(x, nt=128, vt=7, init=0):
    d = np.ascontiguousarray(x, np.int32).copy()
    _check(lib().emu_scan_exc_i32(_ptr(d), d.size, nt, vt, init))
    return d


def emu_radix_sort(keys, vals=None, nt=128, vt=15, num_bits=4):
    k = np.ascontiguousarray(keys).copy()
    v = None if vals is None else np.ascontiguousarray(vals, np.int32).copy()
    _check(lib().emu_radix_sort(EMU_KEYS[k.dtype], _ptr(k), _ptr(v), k.size, nt, vt, num_bits))
    return k, v


def libc_rand(n, seed=1):
    out = np.empty(n, np.uint32)
    lib().emu_libc_rand_fill(_ptr(out), n, seed)
    return out
