"""Python access to libmgpu_gb300.so through its C ABI (include/mgpu_gb300.h).

This is a thin ctypes layer for tests, benchmarks and Python callers.  Device
memory comes from torch (plumbing only); every computation runs in the CUDA
kernels of libmgpu_gb300.so.  There is no CPU fallback: if the library is
missing or fails to load, import of the library raises.
"""
import ctypes
import os

import numpy as np

from . import _lib
from ._lib import MgpuError, lib, library_path  # noqa: F401

DTYPES = {
    np.dtype(np.int32): 0,
    np.dtype(np.uint32): 1,
    np.dtype(np.float32): 2,
    np.dtype(np.int64): 3,
    np.dtype(np.uint64): 4,
    np.dtype(np.float64): 5,
}
SCAN_TYPES = {"exc": 0, "inc": 1}
PRIMITIVES = {"radix": 0, "scan": 1, "merge": 2, "mergesort": 3}
CUDA_STREAM_LEGACY = 0x1    # cudaStreamLegacy: the legacy default stream's handle
OPS = {"plus": 0, "max": 1, "min": 2}
COMPS = {"less": 0, "greater": 1}


def _torch():
    import torch
    return torch


def tuning_variants(primitive, key_dtype):
    """Names of the compiled launch shapes of `primitive` ("radix", "scan",
    "merge", "mergesort") for keys of `key_dtype`, in variant order (host
    only: no device or context needed)."""
    buf = ctypes.create_string_buffer(512)
    n = lib().mgpu_tuning_variants(PRIMITIVES[primitive], DTYPES[np.dtype(key_dtype)], buf, 512)
    return buf.value.decode().split("\n")[:n]


class DeviceArray:
    """A device buffer of `count` elements of a numpy dtype, held by a torch
    uint8 tensor.  Only its pointer is handed to the library."""

    def __init__(self, count, dtype, tensor=None):
        torch = _torch()
        self.dtype = np.dtype(dtype)
        self.count = int(count)
        nbytes = max(1, self.count * self.dtype.itemsize)
        self.tensor = tensor if tensor is not None else torch.empty(
            nbytes, dtype=torch.uint8, device="cuda")

    @classmethod
    def from_numpy(cls, arr, stream=None):
        torch = _torch()
        arr = np.ascontiguousarray(arr)
        out = cls(arr.size, arr.dtype)
        if arr.size:
            host = torch.from_numpy(arr.view(np.uint8).reshape(-1))
            out.tensor[: host.numel()].copy_(host, non_blocking=False)
        return out

    @property
    def ptr(self):
        return self.tensor.data_ptr()

    @property
    def nbytes(self):
        return self.count * self.dtype.itemsize

    def numpy(self):
        if self.count == 0:
            return np.empty(0, self.dtype)
        host = self.tensor[: self.nbytes].cpu().numpy()
        return host.view(self.dtype).copy()

    def copy_from(self, other):
        self.tensor[: self.nbytes].copy_(other.tensor[: other.nbytes])


class Context:
    """mgpu_context_t on one device, enqueuing on torch's current stream of
    that device unless `stream` (a cudaStream_t handle) is given."""

    def __init__(self, device=0, stream=None, use_torch_stream=True):
        torch = _torch()
        if stream is None and use_torch_stream:
            stream = torch.cuda.current_stream(device).cuda_stream
            if stream == 0:
                # torch's default stream is the legacy NULL stream; NULL at the
                # C ABI means "create a private stream", so name it explicitly.
                stream = CUDA_STREAM_LEGACY
        self._h = ctypes.c_void_p()
        _lib.check(lib().mgpu_context_create(device, ctypes.c_void_p(stream), ctypes.byref(self._h)),
                   None)
        self.device = device

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            lib().mgpu_context_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        _lib.check(rc, self._h)

    def synchronize(self):
        self._check(lib().mgpu_synchronize(self._h))

    def set_stream(self, stream):
        self._check(lib().mgpu_context_set_stream(self._h, ctypes.c_void_p(stream)))

    @property
    def sm_count(self):
        return lib().mgpu_sm_count(self._h)

    @property
    def launch_count(self):
        return lib().mgpu_launch_count(self._h)

    def selftest_bounded_wait(self, limit=4096):
        """Enqueues the bounded-wait self test; the next synchronize() raises
        MgpuError with status 3 (a bounded wait gave up)."""
        self._check(lib().mgpu_selftest_bounded_wait(self._h, limit))

    def set_wait_limit(self, polls):
        """Polls before a radix pass's look-back or copy wait gives up (0:
        the library's limit)."""
        self._check(lib().mgpu_set_wait_limit(self._h, polls))

    def selftest_lookback_timeout(self):
        """Runs the production radix pass on a tile whose look-back
        predecessor never publishes (synchronises); the next synchronize()
        raises MgpuError with status 3."""
        self._check(lib().mgpu_selftest_lookback_timeout(self._h))

    # --- launch-shape tuning ---
    def tuning_variants(self, primitive, key_dtype):
        return tuning_variants(primitive, key_dtype)

    def tuning_set(self, primitive, key_dtype, val_bytes, bucket, variant):
        self._check(lib().mgpu_tuning_set(self._h, PRIMITIVES[primitive],
                                          DTYPES[np.dtype(key_dtype)], val_bytes, bucket, variant))

    def tuning_get(self, primitive, key_dtype, val_bytes, count):
        return lib().mgpu_tuning_get(self._h, PRIMITIVES[primitive], DTYPES[np.dtype(key_dtype)],
                                     val_bytes, count)

    def tuning_save(self, path):
        self._check(lib().mgpu_tuning_save(self._h, path.encode()))

    def tuning_load(self, path):
        self._check(lib().mgpu_tuning_load(self._h, path.encode()))

    def autotune(self, primitive, key_dtype, val_bytes, count, reps=3):
        best = ctypes.c_int()
        ms = ctypes.c_double()
        self._check(lib().mgpu_autotune(self._h, PRIMITIVES[primitive],
                                        DTYPES[np.dtype(key_dtype)], val_bytes, count, reps,
                                        ctypes.byref(best), ctypes.byref(ms)))
        return best.value, ms.value

    # --- CUDA graphs ---
    def graph_begin(self):
        self._check(lib().mgpu_graph_begin(self._h))

    def graph_end(self):
        g = ctypes.c_void_p()
        self._check(lib().mgpu_graph_end(self._h, ctypes.byref(g)))
        return Graph(self, g)

    def cache_reserve(self, nbytes):
        self._check(lib().mgpu_cache_reserve(self._h, nbytes))

    # --- profiling ---
    def profile(self, enable=True):
        self._check(lib().mgpu_profile_enable(self._h, int(bool(enable))))

    def profile_read(self):
        cap = 64
        names = ctypes.create_string_buffer(8192)
        launches = (ctypes.c_int64 * cap)()
        total = (ctypes.c_double * cap)()
        num = ctypes.c_int()
        self._check(lib().mgpu_profile_read(self._h, names, 8192, launches, total, cap,
                                            ctypes.byref(num)))
        keys = names.value.decode().split("\n")
        return {keys[i]: (launches[i], total[i]) for i in range(num.value)}

    # --- aux sizing helper: two-phase protocol ---
    @staticmethod
    def _aux_args(aux):
        if aux is None:
            return None, None
        ptr, size = aux
        return ctypes.c_void_p(ptr), ctypes.byref(ctypes.c_size_t(size))

    # --- primitives ---
    def radix_sort_aux_size(self, key_dtype, val_dtype, count):
        size = ctypes.c_size_t(0)
        self._check(lib().mgpu_radix_sort(self._h, DTYPES[np.dtype(key_dtype)], None,
                                          0 if val_dtype is None else np.dtype(val_dtype).itemsize,
                                          None, count, None, ctypes.byref(size)))
        return size.value

    def radix_sort(self, keys, vals=None, aux=None, device_count=None):
        """In-place stable radix sort of DeviceArray keys (and vals).  With
        `device_count` (a device pointer to one int64) the number of keys is
        read on the device when the kernels run; keys.count is the capacity."""
        a, s = self._aux_args(aux)
        vb = 0 if vals is None else vals.dtype.itemsize
        vp = None if vals is None else ctypes.c_void_p(vals.ptr)
        if device_count is None:
            self._check(lib().mgpu_radix_sort(
                self._h, DTYPES[keys.dtype], ctypes.c_void_p(keys.ptr), vb, vp, keys.count, a, s))
        else:
            self._check(lib().mgpu_radix_sort_count_on_device(
                self._h, DTYPES[keys.dtype], ctypes.c_void_p(keys.ptr), vb, vp, keys.count,
                ctypes.c_void_p(device_count), a, s))

    def merge(self, a_keys, a_vals, b_keys, b_vals, c_keys, c_vals, comp="less", aux=None):
        a, s = self._aux_args(aux)
        vb = 0 if a_vals is None else a_vals.dtype.itemsize
        vp = (lambda x: None if x is None else ctypes.c_void_p(x.ptr))
        self._check(lib().mgpu_merge(
            self._h, DTYPES[a_keys.dtype], vp(a_keys), vp(a_vals), a_keys.count,
            vp(b_keys), vp(b_vals), b_keys.count, vp(c_keys), vp(c_vals), vb, COMPS[comp], a, s))

    def mergesort(self, keys, vals=None, comp="less", aux=None):
        a, s = self._aux_args(aux)
        self._check(lib().mgpu_mergesort(
            self._h, DTYPES[keys.dtype], ctypes.c_void_p(keys.ptr),
            0 if vals is None else vals.dtype.itemsize,
            None if vals is None else ctypes.c_void_p(vals.ptr), keys.count, COMPS[comp], a, s))

    def mergesort_indices(self, keys, indices, comp="less", aux=None):
        a, s = self._aux_args(aux)
        self._check(lib().mgpu_mergesort_indices(
            self._h, DTYPES[keys.dtype], ctypes.c_void_p(keys.ptr), ctypes.c_void_p(indices.ptr),
            keys.count, COMPS[comp], a, s))

    def scan(self, data_in, data_out, scan_type="exc", op="plus", init=None, reduction=None,
             aux=None):
        a, s = self._aux_args(aux)
        init_p = None
        if init is not None:
            init_arr = np.array([init], dtype=data_in.dtype)
            init_p = init_arr.ctypes.data_as(ctypes.c_void_p)
        self._check(lib().mgpu_scan(
            self._h, DTYPES[data_in.dtype], SCAN_TYPES[scan_type], OPS[op],
            ctypes.c_void_p(data_in.ptr), ctypes.c_void_p(data_out.ptr), data_in.count, init_p,
            None if reduction is None else ctypes.c_void_p(reduction.ptr), a, s))

    def reduce(self, data_in, out, op="plus", init=None, aux=None):
        a, s = self._aux_args(aux)
        init_p = None
        if init is not None:
            init_arr = np.array([init], dtype=data_in.dtype)
            init_p = init_arr.ctypes.data_as(ctypes.c_void_p)
        self._check(lib().mgpu_reduce(
            self._h, DTYPES[data_in.dtype], OPS[op], ctypes.c_void_p(data_in.ptr), data_in.count,
            init_p, ctypes.c_void_p(out.ptr), a, s))

    def segmented_sort(self, keys, vals, offsets, aux=None):
        a, s = self._aux_args(aux)
        self._check(lib().mgpu_segmented_sort(
            self._h, DTYPES[keys.dtype], ctypes.c_void_p(keys.ptr),
            0 if vals is None else vals.dtype.itemsize,
            None if vals is None else ctypes.c_void_p(vals.ptr), keys.count,
            ctypes.c_void_p(offsets.ptr), offsets.count - 1, a, s))

    def segmented_scan(self, data_in, data_out, offsets, scan_type="inc", op="plus", init=None,
                       aux=None):
        a, s = self._aux_args(aux)
        init_p = None
        if init is not None:
            init_arr = np.array([init], dtype=data_in.dtype)
            init_p = init_arr.ctypes.data_as(ctypes.c_void_p)
        self._check(lib().mgpu_segmented_scan(
            self._h, DTYPES[data_in.dtype], SCAN_TYPES[scan_type], OPS[op],
            ctypes.c_void_p(data_in.ptr), ctypes.c_void_p(data_out.ptr), data_in.count,
            ctypes.c_void_p(offsets.ptr), offsets.count - 1, init_p, a, s))

    def transform_iota(self, out, start=0.0, step=1.0):
        self._check(lib().mgpu_transform_iota(self._h, DTYPES[out.dtype], ctypes.c_void_p(out.ptr),
                                              out.count, float(start), float(step)))

    def transform_fill(self, out, value):
        self._check(lib().mgpu_transform_fill(self._h, DTYPES[out.dtype], ctypes.c_void_p(out.ptr),
                                              out.count, float(value)))

    def transform_saxpy(self, a, x, y):
        self._check(lib().mgpu_transform_saxpy_f32(self._h, ctypes.c_float(a),
                                                   ctypes.c_void_p(x.ptr), ctypes.c_void_p(y.ptr),
                                                   x.count))


class Graph:
    """An executable CUDA graph captured from a context's stream."""

    def __init__(self, ctx, handle):
        self.ctx = ctx
        self._g = handle

    def launch(self):
        self.ctx._check(lib().mgpu_graph_launch(self.ctx.handle, self._g))

    def close(self):
        if self._g:
            lib().mgpu_graph_destroy(self._g)
            self._g = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def build_dir():
    return os.path.dirname(library_path())


class Request(ctypes.Structure):
    """mgpu_request_t."""
    _fields_ = [("op", ctypes.c_int), ("key_type", ctypes.c_int), ("val_bytes", ctypes.c_int),
                ("count", ctypes.c_int64), ("count_b", ctypes.c_int64),
                ("keys", ctypes.c_void_p), ("vals", ctypes.c_void_p),
                ("keys_b", ctypes.c_void_p), ("vals_b", ctypes.c_void_p),
                ("out_keys", ctypes.c_void_p), ("out_vals", ctypes.c_void_p),
                ("scan_type", ctypes.c_int), ("op_arg", ctypes.c_int)]


class ServerStats(ctypes.Structure):
    """mgpu_server_stats_t."""
    _fields_ = [("submitted", ctypes.c_int64), ("completed", ctypes.c_int64),
                ("failed", ctypes.c_int64), ("elements", ctypes.c_int64),
                ("p50_ms", ctypes.c_double), ("p99_ms", ctypes.c_double),
                ("mean_ms", ctypes.c_double), ("max_ms", ctypes.c_double),
                ("peak_bytes", ctypes.c_size_t), ("coalesced", ctypes.c_int64),
                ("batches", ctypes.c_int64)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


REQ_OPS = {"sort": 0, "merge": 1, "scan": 2}


def _host_ptr(a):
    """Address of a C-contiguous numpy array or CPU torch tensor (None -> 0)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        if not a.flags.c_contiguous:
            raise ValueError("host buffers must be C-contiguous")
        return a.ctypes.data
    if a.device.type != "cpu" or not a.is_contiguous():
        raise ValueError("host buffers must be contiguous CPU tensors")
    return a.data_ptr()


def _np_dtype(a):
    if isinstance(a, np.ndarray):
        return a.dtype
    return np.dtype(str(a.dtype).replace("torch.", ""))


class Server:
    """mgpu_server_t: queued sort / merge / scan requests on host buffers,
    admitted under an HBM budget and run concurrently on `num_slots` streams.
    Host buffers are referenced until the request has been waited on; pinned
    buffers (torch `pin_memory()`) give asynchronous copies."""

    def __init__(self, device=0, budget_bytes=8 << 30, num_slots=4):
        self._h = ctypes.c_void_p()
        _lib.check(lib().mgpu_server_create(device, budget_bytes, num_slots,
                                            ctypes.byref(self._h)), None)
        self._held = {}

    def close(self):
        if self._h:
            lib().mgpu_server_destroy(self._h)
            self._h = ctypes.c_void_p()
            self._held.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, req, held=()):
        """Queues a filled-in Request; `held` objects stay referenced until
        the request is waited on."""
        rid = ctypes.c_uint64()
        _lib.check(lib().mgpu_server_submit(self._h, ctypes.byref(req), ctypes.byref(rid)), None)
        self._held[rid.value] = held
        return rid.value

    def submit_sort(self, keys, vals, out_keys, out_vals):
        req = Request(op=0, key_type=DTYPES[_np_dtype(keys)],
                      val_bytes=0 if vals is None else _np_dtype(vals).itemsize,
                      count=len(keys), keys=_host_ptr(keys), vals=_host_ptr(vals),
                      out_keys=_host_ptr(out_keys), out_vals=_host_ptr(out_vals))
        return self.submit(req, (keys, vals, out_keys, out_vals))

    def submit_merge(self, a_keys, a_vals, b_keys, b_vals, out_keys, out_vals, comp="less"):
        req = Request(op=1, key_type=DTYPES[_np_dtype(a_keys)],
                      val_bytes=0 if a_vals is None else _np_dtype(a_vals).itemsize,
                      count=len(a_keys), count_b=len(b_keys),
                      keys=_host_ptr(a_keys), vals=_host_ptr(a_vals),
                      keys_b=_host_ptr(b_keys), vals_b=_host_ptr(b_vals),
                      out_keys=_host_ptr(out_keys), out_vals=_host_ptr(out_vals),
                      op_arg=COMPS[comp])
        return self.submit(req, (a_keys, a_vals, b_keys, b_vals, out_keys, out_vals))

    def submit_scan(self, data, out, scan_type="exc", op="plus"):
        req = Request(op=2, key_type=DTYPES[_np_dtype(data)], count=len(data),
                      keys=_host_ptr(data), out_keys=_host_ptr(out),
                      scan_type=SCAN_TYPES[scan_type], op_arg=OPS[op])
        return self.submit(req, (data, out))

    def poll(self, rid):
        """True when done (releases the id), False while queued or running."""
        rc = lib().mgpu_server_poll(self._h, rid)
        if rc == 7:
            return False
        self._held.pop(rid, None)
        _lib.check(rc, None)
        return True

    def wait(self, rid):
        """Blocks until the request is done; returns its latency in ms."""
        lat = ctypes.c_double()
        rc = lib().mgpu_server_wait(self._h, rid, ctypes.byref(lat))
        self._held.pop(rid, None)
        _lib.check(rc, None)
        return lat.value

    def drain(self):
        _lib.check(lib().mgpu_server_drain(self._h), None)

    def stats(self):
        s = ServerStats()
        _lib.check(lib().mgpu_server_stats(self._h, ctypes.byref(s)), None)
        return s.as_dict()

    def reset_stats(self):
        _lib.check(lib().mgpu_server_reset_stats(self._h), None)
