"""PyTorch operators over the C ABI (include/mgpu_gb300.h).

Importing this module registers, with torch.library:

    torch.ops.mgpu.radix_sort_(keys, values)                 in place, stable
    torch.ops.mgpu.sort_(keys, values, descending=False)      in place, stable
    torch.ops.mgpu.merge(a_keys, a_values, b_keys, b_values, descending=False)
                                                -> (keys, values)
    torch.ops.mgpu.merge_keys(a_keys, b_keys, descending=False) -> keys
    torch.ops.mgpu.scan(x, inclusive=False, op="plus") -> Tensor
    torch.ops.mgpu.segmented_sort_(keys, values, offsets)      in place
    torch.ops.mgpu.segmented_scan(x, offsets, inclusive=True, op="plus") -> Tensor

Tensors are 1-D, contiguous and on a CUDA device; keys int32, uint32,
float32, int64, uint64 or float64; values 4 or 8 bytes per element; offsets
int64 (num_segments + 1 entries, CSR).  `values` may be None (keys only); it
has no default because an in-place operator's optional tensors are passed
explicitly.  Work is enqueued on torch's current
stream of the tensors' device, without a host synchronisation, through one
library context per (device, stream); `synchronize()` waits for those
streams and raises if a kernel reported an error.  radix_sort_ orders floats
by their bits (-0.0 before +0.0, NaNs by bit pattern), as the library's
radix sort does; sort_ and merge compare with < (or >).  There is no CPU
path: a CPU tensor is an error.
"""
import ctypes
from typing import Optional, Tuple

import torch

from . import _lib
from ._lib import lib

_DTYPE_CODES = {torch.int32: 0, torch.float32: 2, torch.int64: 3, torch.float64: 5}
if hasattr(torch, "uint32"):
    _DTYPE_CODES[torch.uint32] = 1
if hasattr(torch, "uint64"):
    _DTYPE_CODES[torch.uint64] = 4
_OPS = {"plus": 0, "max": 1, "min": 2}
_CUDA_STREAM_LEGACY = 0x1

_contexts = {}


def _context(device):
    """The library context bound to torch's current stream on `device`."""
    stream = torch.cuda.current_stream(device).cuda_stream or _CUDA_STREAM_LEGACY
    key = (device.index, stream)
    h = _contexts.get(key)
    if h is None:
        h = ctypes.c_void_p()
        _lib.check(lib().mgpu_context_create(device.index, ctypes.c_void_p(stream),
                                             ctypes.byref(h)), None)
        _contexts[key] = h
    return h


def synchronize():
    """Waits for every stream an operator was enqueued on; raises MgpuError
    if a kernel reported an error (a bounded wait that gave up)."""
    for h in _contexts.values():
        _lib.check(lib().mgpu_synchronize(h), h)


def _code(t, what):
    if t.device.type != "cuda":
        raise ValueError("%s must be a CUDA tensor (there is no CPU path)" % what)
    if t.dim() != 1 or not t.is_contiguous():
        raise ValueError("%s must be a contiguous 1-D tensor" % what)
    code = _DTYPE_CODES.get(t.dtype)
    if code is None:
        raise ValueError("%s: unsupported dtype %s" % (what, t.dtype))
    return code


def _values(values, keys):
    if values is None:
        return 0, None
    if values.device != keys.device or values.dim() != 1 or not values.is_contiguous():
        raise ValueError("values must be a contiguous 1-D tensor on the keys' device")
    if values.numel() != keys.numel():
        raise ValueError("values and keys differ in length")
    if values.element_size() not in (4, 8):
        raise ValueError("values must have 4 or 8 bytes per element")
    return values.element_size(), ctypes.c_void_p(values.data_ptr())


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _offsets(offsets, keys):
    if offsets.dtype != torch.int64 or offsets.device != keys.device or offsets.dim() != 1 \
            or not offsets.is_contiguous() or offsets.numel() < 2:
        raise ValueError("offsets must be a contiguous 1-D int64 tensor of num_segments + 1 "
                         "entries on the keys' device")
    return offsets.numel() - 1


@torch.library.custom_op("mgpu::radix_sort_", mutates_args=("keys", "values"))
def radix_sort_(keys: torch.Tensor, values: Optional[torch.Tensor]) -> None:
    code = _code(keys, "keys")
    vb, vp = _values(values, keys)
    h = _context(keys.device)
    _lib.check(lib().mgpu_radix_sort(h, code, _ptr(keys), vb, vp, keys.numel(), None, None), h)


@radix_sort_.register_fake
def _(keys, values):
    return None


@torch.library.custom_op("mgpu::sort_", mutates_args=("keys", "values"))
def sort_(keys: torch.Tensor, values: Optional[torch.Tensor], descending: bool = False) -> None:
    code = _code(keys, "keys")
    vb, vp = _values(values, keys)
    h = _context(keys.device)
    _lib.check(lib().mgpu_mergesort(h, code, _ptr(keys), vb, vp, keys.numel(),
                                    1 if descending else 0, None, None), h)


@sort_.register_fake
def _(keys, values, descending=False):
    return None


def _merge_check(a, b):
    code = _code(a, "a_keys")
    if _code(b, "b_keys") != code or b.device != a.device:
        raise ValueError("a_keys and b_keys must share dtype and device")
    return code


@torch.library.custom_op("mgpu::merge", mutates_args=())
def merge(a_keys: torch.Tensor, a_values: torch.Tensor, b_keys: torch.Tensor,
          b_values: torch.Tensor, descending: bool = False) -> Tuple[torch.Tensor, torch.Tensor]:
    code = _merge_check(a_keys, b_keys)
    vb, avp = _values(a_values, a_keys)
    vb2, bvp = _values(b_values, b_keys)
    if vb != vb2 or a_values.dtype != b_values.dtype:
        raise ValueError("a_values and b_values must share dtype")
    n = a_keys.numel() + b_keys.numel()
    c_keys = torch.empty(n, dtype=a_keys.dtype, device=a_keys.device)
    c_vals = torch.empty(n, dtype=a_values.dtype, device=a_keys.device)
    h = _context(a_keys.device)
    _lib.check(lib().mgpu_merge(h, code, _ptr(a_keys), avp, a_keys.numel(), _ptr(b_keys), bvp,
                                b_keys.numel(), _ptr(c_keys), _ptr(c_vals), vb,
                                1 if descending else 0, None, None), h)
    return c_keys, c_vals


@merge.register_fake
def _(a_keys, a_values, b_keys, b_values, descending=False):
    n = a_keys.numel() + b_keys.numel()
    return a_keys.new_empty(n), a_values.new_empty(n)


@torch.library.custom_op("mgpu::merge_keys", mutates_args=())
def merge_keys(a_keys: torch.Tensor, b_keys: torch.Tensor,
               descending: bool = False) -> torch.Tensor:
    code = _merge_check(a_keys, b_keys)
    c_keys = torch.empty(a_keys.numel() + b_keys.numel(), dtype=a_keys.dtype,
                         device=a_keys.device)
    h = _context(a_keys.device)
    _lib.check(lib().mgpu_merge(h, code, _ptr(a_keys), None, a_keys.numel(), _ptr(b_keys), None,
                                b_keys.numel(), _ptr(c_keys), None, 0,
                                1 if descending else 0, None, None), h)
    return c_keys


@merge_keys.register_fake
def _(a_keys, b_keys, descending=False):
    return a_keys.new_empty(a_keys.numel() + b_keys.numel())


@torch.library.custom_op("mgpu::scan", mutates_args=())
def scan(x: torch.Tensor, inclusive: bool = False, op: str = "plus") -> torch.Tensor:
    code = _code(x, "x")
    if op not in _OPS:
        raise ValueError("op must be one of %s" % sorted(_OPS))
    out = torch.empty_like(x)
    h = _context(x.device)
    _lib.check(lib().mgpu_scan(h, code, 1 if inclusive else 0, _OPS[op], _ptr(x), _ptr(out),
                               x.numel(), None, None, None, None), h)
    return out


@scan.register_fake
def _(x, inclusive=False, op="plus"):
    return torch.empty_like(x)


@torch.library.custom_op("mgpu::segmented_sort_", mutates_args=("keys", "values"))
def segmented_sort_(keys: torch.Tensor, values: Optional[torch.Tensor],
                    offsets: torch.Tensor) -> None:
    code = _code(keys, "keys")
    vb, vp = _values(values, keys)
    num_segments = _offsets(offsets, keys)
    h = _context(keys.device)
    _lib.check(lib().mgpu_segmented_sort(h, code, _ptr(keys), vb, vp, keys.numel(),
                                         _ptr(offsets), num_segments, None, None), h)


@segmented_sort_.register_fake
def _(keys, values, offsets):
    return None


@torch.library.custom_op("mgpu::segmented_scan", mutates_args=())
def segmented_scan(x: torch.Tensor, offsets: torch.Tensor, inclusive: bool = True,
                   op: str = "plus") -> torch.Tensor:
    code = _code(x, "x")
    if op not in _OPS:
        raise ValueError("op must be one of %s" % sorted(_OPS))
    num_segments = _offsets(offsets, x)
    out = torch.empty_like(x)
    h = _context(x.device)
    _lib.check(lib().mgpu_segmented_scan(h, code, 1 if inclusive else 0, _OPS[op], _ptr(x),
                                         _ptr(out), x.numel(), _ptr(offsets), num_segments,
                                         None, None, None), h)
    return out


@segmented_scan.register_fake
def _(x, offsets, inclusive=True, op="plus"):
    return torch.empty_like(x)


__all__ = ["radix_sort_", "sort_", "merge", "merge_keys", "scan", "segmented_sort_",
           "segmented_scan", "synchronize"]
