"""Loader and prototypes of libmgpu_gb300.so (the C ABI in include/mgpu_gb300.h)."""
import ctypes
import os
import re

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REPO = os.path.dirname(PKG)
HEADER = os.path.join(REPO, "include", "mgpu_gb300.h")

_lib = None


class MgpuError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(message)
        self.status = status


def library_path():
    return os.path.join(PKG, "lib", "libmgpu_gb300.so")


def declared_functions():
    """Names of the functions declared in include/mgpu_gb300.h."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mgpu_[a-z0-9_]+)\s*\(", text)))


_VP, _I64, _I32, _SZ = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_void_p
_SIGS = {
    "mgpu_context_create": ([_I32, _VP, _VP], _I32),
    "mgpu_context_destroy": ([_VP], _I32),
    "mgpu_context_set_stream": ([_VP, _VP], _I32),
    "mgpu_context_stream": ([_VP], _VP),
    "mgpu_synchronize": ([_VP], _I32),
    "mgpu_status_string": ([_I32], ctypes.c_char_p),
    "mgpu_last_error": ([_VP], ctypes.c_char_p),
    "mgpu_sm_count": ([_VP], _I32),
    "mgpu_alloc_gpu": ([_VP, ctypes.c_size_t, _VP], _I32),
    "mgpu_alloc_cpu": ([_VP, ctypes.c_size_t, _VP], _I32),
    "mgpu_free": ([_VP, _VP], _I32),
    "mgpu_memcpy": ([_VP, _VP, _VP, ctypes.c_size_t], _I32),
    "mgpu_memset": ([_VP, _VP, _I32, ctypes.c_size_t], _I32),
    "mgpu_radix_sort": ([_VP, _I32, _VP, _I32, _VP, _I64, _VP, _SZ], _I32),
    "mgpu_radix_sort_count_on_device": ([_VP, _I32, _VP, _I32, _VP, _I64, _VP, _VP, _SZ], _I32),
    "mgpu_merge": ([_VP, _I32, _VP, _VP, _I64, _VP, _VP, _I64, _VP, _VP, _I32, _I32, _VP, _SZ],
                   _I32),
    "mgpu_mergesort": ([_VP, _I32, _VP, _I32, _VP, _I64, _I32, _VP, _SZ], _I32),
    "mgpu_mergesort_indices": ([_VP, _I32, _VP, _VP, _I64, _I32, _VP, _SZ], _I32),
    "mgpu_scan": ([_VP, _I32, _I32, _I32, _VP, _VP, _I64, _VP, _VP, _VP, _SZ], _I32),
    "mgpu_reduce": ([_VP, _I32, _I32, _VP, _I64, _VP, _VP, _VP, _SZ], _I32),
    "mgpu_transform_iota": ([_VP, _I32, _VP, _I64, ctypes.c_double, ctypes.c_double], _I32),
    "mgpu_transform_fill": ([_VP, _I32, _VP, _I64, ctypes.c_double], _I32),
    "mgpu_transform_saxpy_f32": ([_VP, ctypes.c_float, _VP, _VP, _I64], _I32),
    "mgpu_segmented_sort": ([_VP, _I32, _VP, _I32, _VP, _I64, _VP, _I64, _VP, _SZ], _I32),
    "mgpu_segmented_scan": ([_VP, _I32, _I32, _I32, _VP, _VP, _I64, _VP, _I64, _VP, _VP, _SZ],
                            _I32),
    "mgpu_tuning_variants": ([_I32, _I32, _VP, ctypes.c_size_t], _I32),
    "mgpu_tuning_set": ([_VP, _I32, _I32, _I32, _I32, _I32], _I32),
    "mgpu_tuning_get": ([_VP, _I32, _I32, _I32, _I64], _I32),
    "mgpu_tuning_save": ([_VP, ctypes.c_char_p], _I32),
    "mgpu_tuning_load": ([_VP, ctypes.c_char_p], _I32),
    "mgpu_autotune": ([_VP, _I32, _I32, _I32, _I64, _I32, _VP, _VP], _I32),
    "mgpu_graph_begin": ([_VP], _I32),
    "mgpu_graph_end": ([_VP, _VP], _I32),
    "mgpu_graph_launch": ([_VP, _VP], _I32),
    "mgpu_graph_destroy": ([_VP], _I32),
    "mgpu_cache_reserve": ([_VP, ctypes.c_size_t], _I32),
    "mgpu_server_create": ([_I32, ctypes.c_size_t, _I32, _VP], _I32),
    "mgpu_server_submit": ([_VP, _VP, _VP], _I32),
    "mgpu_server_poll": ([_VP, ctypes.c_uint64], _I32),
    "mgpu_server_wait": ([_VP, ctypes.c_uint64, _VP], _I32),
    "mgpu_server_drain": ([_VP], _I32),
    "mgpu_server_stats": ([_VP, _VP], _I32),
    "mgpu_server_reset_stats": ([_VP], _I32),
    "mgpu_server_destroy": ([_VP], _I32),
    "mgpu_profile_enable": ([_VP, _I32], _I32),
    "mgpu_profile_read": ([_VP, _VP, ctypes.c_size_t, _VP, _VP, _I32, _VP], _I32),
    "mgpu_launch_count": ([_VP], _I64),
    "mgpu_selftest_bounded_wait": ([_VP, _I32], _I32),
    "mgpu_selftest_lookback_timeout": ([_VP], _I32),
    "mgpu_set_wait_limit": ([_VP, _I32], _I32),
    "mgpu_scan_noalloc": ([_VP, _I32, _I32, _I32, _VP, _VP, _I64, _VP, _VP], _I32),
    "mgpu_scan_noalloc_status": ([_VP], _I32),
    "mgpu_selftest_scan_noalloc_wait": ([_VP, _I32], _I32),
}


def lib(path=None):
    """Loads the library (building it first if it is absent) and sets the
    prototypes.  Raises if it cannot be loaded: there is no fallback."""
    global _lib
    if _lib is None:
        path = path or library_path()
        if not os.path.exists(path):
            import importlib.util
            spec = importlib.util.spec_from_file_location("_mgpu_build",
                                                          os.path.join(PKG, "build.py"))
            mod = importlib.util.module_from_spec(spec)
            spec.loader.exec_module(mod)
            mod.build()
        handle = ctypes.CDLL(path)
        for name, (args, res) in _SIGS.items():
            f = getattr(handle, name, None)
            if f is None:
                continue
            f.argtypes = args
            f.restype = res
        _lib = handle
    return _lib


def check(rc, ctx):
    if rc != 0:
        msg = lib().mgpu_status_string(rc).decode()
        if ctx is not None and ctx:
            detail = lib().mgpu_last_error(ctx)
            if detail:
                msg += " (" + detail.decode() + ")"
        raise MgpuError(rc, msg)
