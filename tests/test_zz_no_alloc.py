"""mgpu_scan_noalloc: the scan for callers that cannot allocate device memory
(an engine that owns all device memory, a plugin whose enqueue must not
allocate, a pipeline that forbids allocation after start-up).  It is called
here through the C ABI and compared with the existing entry point, mgpu_scan,
on two calls in a row: the second call must not see anything the first left
in the shared scratch array.  Integers must match exactly; float32 within the
same bound the scan tests use against the float64 oracle.

This file is collected last so that a run stopping at the first failure has
already run every other test; it also passes alone in a fresh process."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

F32_REL = 1e-4
F32_ABS = 1e-6
CODES = {np.dtype(np.int32): 0, np.dtype(np.uint32): 1, np.dtype(np.float32): 2}
SCAN = {"exc": 0, "inc": 1}
OPS = {"plus": 0, "max": 1, "min": 2}


def noalloc_fn(mgpu):
    f = mgpu.lib().mgpu_scan_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                  ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


def run_noalloc(mgpu, x, scan_type, op):
    import torch
    fn = noalloc_fn(mgpu)
    d = mgpu.DeviceArray.from_numpy(x)
    out = mgpu.DeviceArray(x.size, x.dtype)
    red = mgpu.DeviceArray(1, x.dtype)
    stream = torch.cuda.current_stream().cuda_stream
    rc = fn(ctypes.c_void_p(stream), CODES[x.dtype], SCAN[scan_type], OPS[op],
            ctypes.c_void_p(d.ptr), ctypes.c_void_p(out.ptr), x.size, None,
            ctypes.c_void_p(red.ptr))
    assert rc == 0
    torch.cuda.synchronize()
    return out.numpy(), red.numpy()[0]


def run_existing(mgpu, ctx, x, scan_type, op):
    d = mgpu.DeviceArray.from_numpy(x)
    out = mgpu.DeviceArray(x.size, x.dtype)
    red = mgpu.DeviceArray(1, x.dtype)
    ctx.scan(d, out, scan_type=scan_type, op=op, reduction=red)
    ctx.synchronize()
    return out.numpy(), red.numpy()[0]


@pytest.mark.parametrize("dt,scan_type,op", [
    (np.int32, "exc", "plus"), (np.uint32, "inc", "max"), (np.int32, "inc", "min"),
])
def test_noalloc_matches_scan_twice_integers(mgpu, ctx, dt, scan_type, op):
    rng = np.random.default_rng(11)
    # A large call, then a smaller one: the second reuses the scratch words the
    # first filled, which each call clears before its kernel runs.
    for n in (3_000_017, 70_001):
        x = rng.integers(0, 1000, n).astype(dt)
        got, got_red = run_noalloc(mgpu, x, scan_type, op)
        ref, ref_red = run_existing(mgpu, ctx, x, scan_type, op)
        assert np.array_equal(got, ref)
        assert got_red == ref_red


def test_noalloc_matches_scan_twice_float32(mgpu, ctx, oracle):
    rng = np.random.default_rng(12)
    for n in (1_000_003, 4097):
        x = rng.standard_normal(n).astype(np.float32)
        got, _ = run_noalloc(mgpu, x, "inc", "plus")
        ref, _ = run_existing(mgpu, ctx, x, "inc", "plus")
        _, ref_abs = oracle.scan_fp(x, exclusive=False)
        bound = F32_REL * ref_abs + F32_ABS
        assert np.all(np.abs(got.astype(np.float64) - ref.astype(np.float64)) <= bound)


def test_noalloc_rejects_sizes_beyond_its_scratch(mgpu):
    import torch
    fn = noalloc_fn(mgpu)
    stream = torch.cuda.current_stream().cuda_stream
    # Rejected on the host before anything is enqueued.
    rc = fn(ctypes.c_void_p(stream), 0, 0, 0, None, None, (1 << 28) + 1, None, None)
    assert rc == 1   # MGPU_ERR_INVALID_ARG
