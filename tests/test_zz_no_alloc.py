"""mgpu_scan_noalloc: the scan for callers that cannot allocate device memory
(an engine that owns all device memory, a plugin whose enqueue must not
allocate, a pipeline that forbids allocation after start-up).  It is called
here through the C ABI and compared with the existing entry point, mgpu_scan,
on two calls in a row: the second call must not see anything the first left
in the shared scratch array.  Integers must match exactly; float32 within the
same bound the scan tests use against the float64 oracle.  Every call's
returned status and the device-side status (mgpu_scan_noalloc_status) are
checked, including a wait that gives up on purpose (a flag nothing sets, a
short poll limit: no fault).

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
MAX_COUNT = 1 << 28          # MGPU_SCAN_NOALLOC_MAX_COUNT


def _stream():
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _init_ptr(init, dtype):
    if init is None:
        return None, None
    arr = np.array([init], dtype=dtype)
    return arr, arr.ctypes.data_as(ctypes.c_void_p)


def noalloc(mgpu, d_in, d_out, count, dtype, scan_type, op, init=None, red=None):
    """One mgpu_scan_noalloc call on torch's current stream; returns its status."""
    keep, init_p = _init_ptr(init, dtype)
    rc = mgpu.lib().mgpu_scan_noalloc(
        _stream(), CODES[np.dtype(dtype)], SCAN[scan_type], OPS[op],
        ctypes.c_void_p(d_in.ptr) if d_in is not None else None,
        ctypes.c_void_p(d_out.ptr) if d_out is not None else None, count, init_p,
        ctypes.c_void_p(red.ptr) if red is not None else None)
    del keep
    return rc


def device_status(mgpu):
    return mgpu.lib().mgpu_scan_noalloc_status(_stream())


def run_noalloc(mgpu, x, scan_type, op, init=None):
    import torch
    d = mgpu.DeviceArray.from_numpy(x)
    out = mgpu.DeviceArray(x.size, x.dtype)
    red = mgpu.DeviceArray(1, x.dtype)
    assert noalloc(mgpu, d, out, x.size, x.dtype, scan_type, op, init, red) == 0
    torch.cuda.synchronize()
    assert device_status(mgpu) == 0
    return out.numpy(), red.numpy()[0]


def run_existing(mgpu, ctx, x, scan_type, op, init=None):
    d = mgpu.DeviceArray.from_numpy(x)
    out = mgpu.DeviceArray(x.size, x.dtype)
    red = mgpu.DeviceArray(1, x.dtype)
    ctx.scan(d, out, scan_type=scan_type, op=op, init=init, reduction=red)
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


@pytest.mark.parametrize("dt,scan_type,op,init", [
    (np.int32, "exc", "plus", 7), (np.int32, "inc", "plus", -123456),
    (np.uint32, "inc", "max", 500), (np.int32, "exc", "min", 10),
])
def test_noalloc_with_init_matches_scan_and_oracle(mgpu, ctx, oracle, dt, scan_type, op, init):
    rng = np.random.default_rng(13)
    x = rng.integers(0, 1000, 500_009).astype(dt)
    got, got_red = run_noalloc(mgpu, x, scan_type, op, init)
    ref, ref_red = run_existing(mgpu, ctx, x, scan_type, op, init)
    assert np.array_equal(got, ref)
    assert got_red == ref_red
    if op == "plus" and dt == np.int32:
        expect = oracle.scan_int(x, exclusive=(scan_type == "exc")).astype(np.int64) + init
        assert np.array_equal(got, (expect & 0xFFFFFFFF).astype(np.uint32).view(np.int32))


def test_noalloc_unaligned_views_take_the_scalar_path(mgpu, ctx, oracle):
    """in and out 4 bytes past a 16-byte boundary: no 16-byte vector access."""
    import torch
    rng = np.random.default_rng(14)
    n = 1_000_003
    x = rng.integers(-50, 50, n).astype(np.int32)
    base_in = mgpu.DeviceArray.from_numpy(np.concatenate([np.zeros(1, np.int32), x]))
    base_out = mgpu.DeviceArray(n + 1, np.int32)
    d_in = mgpu.DeviceArray(n, np.int32, tensor=base_in.tensor[4:])
    d_out = mgpu.DeviceArray(n, np.int32, tensor=base_out.tensor[4:])
    assert d_in.ptr % 16 != 0 and d_out.ptr % 16 != 0
    for scan_type in ("exc", "inc"):
        assert noalloc(mgpu, d_in, d_out, n, np.int32, scan_type, "plus") == 0
        torch.cuda.synchronize()
        assert device_status(mgpu) == 0
        assert np.array_equal(d_out.numpy(), oracle.scan_int(x, exclusive=(scan_type == "exc")))
        ref, _ = run_existing(mgpu, ctx, x, scan_type, "plus")
        assert np.array_equal(d_out.numpy(), ref)


def test_noalloc_in_place(mgpu, ctx, oracle):
    """in == out: the reference's vk::scan form (it scans in place)."""
    import torch
    rng = np.random.default_rng(15)
    for n in (2_000_001, 4096):
        x = rng.integers(0, 100, n).astype(np.int32)
        d = mgpu.DeviceArray.from_numpy(x)
        red = mgpu.DeviceArray(1, np.int32)
        assert noalloc(mgpu, d, d, n, np.int32, "exc", "plus", None, red) == 0
        torch.cuda.synchronize()
        assert device_status(mgpu) == 0
        ref, ref_red = run_existing(mgpu, ctx, x, "exc", "plus")
        assert np.array_equal(d.numpy(), ref)
        assert np.array_equal(d.numpy(), oracle.scan_int(x, exclusive=True))
        assert red.numpy()[0] == ref_red


def test_noalloc_count_zero_writes_the_reduction(mgpu):
    import torch
    red = mgpu.DeviceArray.from_numpy(np.array([99], np.int32))
    assert noalloc(mgpu, None, None, 0, np.int32, "exc", "plus", 42, red) == 0
    torch.cuda.synchronize()
    assert red.numpy()[0] == 42
    red_max = mgpu.DeviceArray.from_numpy(np.array([99], np.int32))
    assert noalloc(mgpu, None, None, 0, np.int32, "inc", "max", None, red_max) == 0
    torch.cuda.synchronize()
    assert red_max.numpy()[0] == np.iinfo(np.int32).min
    assert device_status(mgpu) == 0


@pytest.mark.slow
def test_noalloc_at_its_maximum_count(mgpu, ctx):
    """Exactly MGPU_SCAN_NOALLOC_MAX_COUNT elements (every scratch word used),
    in place, against mgpu_scan of a copy; compared on the device."""
    import torch
    g = torch.Generator(device="cuda")
    g.manual_seed(16)
    src = torch.randint(0, 100, (MAX_COUNT,), dtype=torch.int32, device="cuda", generator=g)
    work = src.clone()
    ref = torch.empty_like(src)
    d_work = mgpu.DeviceArray(MAX_COUNT, np.int32, tensor=work.view(torch.uint8))
    d_src = mgpu.DeviceArray(MAX_COUNT, np.int32, tensor=src.view(torch.uint8))
    d_ref = mgpu.DeviceArray(MAX_COUNT, np.int32, tensor=ref.view(torch.uint8))
    red = mgpu.DeviceArray(1, np.int32)
    ref_red = mgpu.DeviceArray(1, np.int32)
    for scan_type in ("inc", "exc"):
        work.copy_(src)
        assert noalloc(mgpu, d_work, d_work, MAX_COUNT, np.int32, scan_type, "plus", None,
                       red) == 0
        ctx.scan(d_src, d_ref, scan_type=scan_type, reduction=ref_red)
        ctx.synchronize()
        torch.cuda.synchronize()
        assert device_status(mgpu) == 0
        assert torch.equal(work, ref)
        assert red.numpy()[0] == ref_red.numpy()[0]
    del work, ref, src
    torch.cuda.empty_cache()


def test_noalloc_rejects_sizes_beyond_its_scratch(mgpu):
    # Rejected on the host before anything is enqueued.
    assert noalloc(mgpu, None, None, MAX_COUNT + 1, np.int32, "exc", "plus") == 1
    assert noalloc(mgpu, None, None, -1, np.int32, "exc", "plus") == 1


def test_noalloc_status_reports_a_wait_that_gave_up(mgpu, ctx):
    """A bounded wait that gives up is reported once by the status query, which
    clears it; scans afterwards are right again."""
    import torch
    lib = mgpu.lib()
    assert device_status(mgpu) == 0
    assert lib.mgpu_selftest_scan_noalloc_wait(_stream(), 0) == 1       # limit checked
    assert lib.mgpu_selftest_scan_noalloc_wait(_stream(), 2048) == 0
    torch.cuda.synchronize()
    assert device_status(mgpu) == 3          # MGPU_ERR_LOOKBACK_TIMEOUT
    assert device_status(mgpu) == 0          # read and cleared
    rng = np.random.default_rng(17)
    x = rng.integers(0, 1000, 300_007).astype(np.int32)
    got, _ = run_noalloc(mgpu, x, "inc", "plus")
    ref, _ = run_existing(mgpu, ctx, x, "inc", "plus")
    assert np.array_equal(got, ref)
