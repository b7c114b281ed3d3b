"""Parity of mgpu_scan / mgpu_reduce (single-pass look-back, sm_103a) with the
host oracle.  Integer scans are bit-exact with two's-complement wrap (the
reference's 32-bit GPU adds, vk/scan.hxx:10-115).  Float scans are checked
against a float64 oracle with a bound scaled by the prefix of |x|."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# Per-element bound of a float32 scan against the float64 oracle:
#   |gpu_i - ref_i| <= F32_REL * sum_{j<=i} |x_j| + F32_ABS
F32_REL = 1e-4
F32_ABS = 1e-6
F64_REL = 1e-12

SIZES = [0, 1, 2, 31, 32, 33, 4095, 4096, 4097, 2 * 4096 + 3, 100_000, 1_000_003]
INT_TYPES = [np.int32, np.uint32, np.int64, np.uint64]


def run_scan(mgpu, ctx, x, scan_type, op="plus", init=None, in_place=False):
    d = mgpu.DeviceArray.from_numpy(x)
    out = d if in_place else mgpu.DeviceArray(x.size, x.dtype)
    red = mgpu.DeviceArray(1, x.dtype)
    ctx.scan(d, out, scan_type=scan_type, op=op, init=init, reduction=red)
    ctx.synchronize()
    return out.numpy(), red.numpy()[0]


def ints(rng, n, dt, lo=0, hi=100):
    return rng.integers(lo, hi, n).astype(dt)


@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("scan_type", ["exc", "inc"])
def test_scan_int32_sizes(mgpu, ctx, oracle, rng, n, scan_type):
    x = ints(rng, n, np.int32)
    got, red = run_scan(mgpu, ctx, x, scan_type)
    ref = oracle.scan_int(x, exclusive=scan_type == "exc")
    assert np.array_equal(got, ref)
    assert red == (np.int64(x.astype(np.int64).sum()) & 0xFFFFFFFF).astype(np.uint32).view(np.int32)


@pytest.mark.parametrize("dt", INT_TYPES)
@pytest.mark.parametrize("op", ["plus", "max", "min"])
@pytest.mark.parametrize("scan_type", ["exc", "inc"])
def test_scan_int_ops(mgpu, ctx, oracle, rng, dt, op, scan_type):
    n = 300_007
    info = np.iinfo(dt)
    x = rng.integers(max(info.min, -2 ** 40), min(info.max, 2 ** 40), n).astype(dt)
    init = dt(5) if op == "plus" else None
    got, _ = run_scan(mgpu, ctx, x, scan_type, op=op, init=init)
    kw = {} if init is None else {"init": init}
    if init is None and op != "plus":
        kw["init"] = {"max": info.min, "min": info.max}[op]
    ref = oracle.scan_int(x, exclusive=scan_type == "exc", op=op, **kw)
    assert np.array_equal(got, ref)


def test_scan_in_place_reference_default(mgpu, ctx, oracle, rng):
    """vk::scan's own call shape: exclusive, in place, init = 0
    (examples/vk_scan/vk_scan.cxx: host[i] = i -> i(i-1)/2)."""
    n = 10000
    x = np.arange(n, dtype=np.int32)
    got, _ = run_scan(mgpu, ctx, x, "exc", in_place=True)
    expect = (np.arange(n, dtype=np.int64) * (np.arange(n) - 1) // 2).astype(np.int32)
    assert np.array_equal(got, expect)


def test_scan_int32_wraps(mgpu, ctx, oracle, rng):
    """The 2^28 U[0,100) sum exceeds 2^31; the GPU wraps exactly like the
    oracle's uint32 accumulation."""
    n = 50_000_000
    x = ints(rng, n, np.int32)
    got, _ = run_scan(mgpu, ctx, x, "inc")
    ref = oracle.scan_int(x, exclusive=False)
    assert np.array_equal(got, ref)
    assert x.astype(np.int64).sum() > 2 ** 31


@pytest.mark.parametrize("n", [1, 4097, 1_000_003])
@pytest.mark.parametrize("scan_type", ["exc", "inc"])
def test_scan_f32_tolerance(mgpu, ctx, oracle, rng, n, scan_type):
    x = rng.standard_normal(n).astype(np.float32)
    got, red = run_scan(mgpu, ctx, x, scan_type)
    ref, ref_abs = oracle.scan_fp(x, exclusive=scan_type == "exc")
    err = np.abs(got.astype(np.float64) - ref)
    bound = F32_REL * ref_abs + F32_ABS
    assert np.all(err <= bound), float(np.max(err / bound))


def test_scan_f64(mgpu, ctx, oracle, rng):
    n = 500_001
    x = rng.standard_normal(n)
    got, _ = run_scan(mgpu, ctx, x, "inc")
    ref, ref_abs = oracle.scan_fp(x, exclusive=False)
    assert np.all(np.abs(got - ref) <= F64_REL * ref_abs + 1e-12)


@pytest.mark.parametrize("dt", [np.int32, np.uint64, np.float32, np.float64])
@pytest.mark.parametrize("op", ["plus", "max", "min"])
@pytest.mark.parametrize("n", [0, 1, 1000, 2_000_001])
def test_reduce(mgpu, ctx, rng, dt, op, n):
    if np.dtype(dt).kind == "f":
        x = rng.standard_normal(n).astype(dt)
    else:
        x = rng.integers(0, 1000, n).astype(dt)
    d = mgpu.DeviceArray.from_numpy(x)
    out = mgpu.DeviceArray(1, dt)
    init = dt(3)
    ctx.reduce(d, out, op=op, init=init)
    ctx.synchronize()
    got = out.numpy()[0]
    if op == "plus":
        ref = x.astype(np.float64).sum() + 3 if np.dtype(dt).kind == "f" else \
            (x.astype(np.uint64).sum() + 3).astype(dt)
    elif op == "max":
        ref = max(x.max(), init) if n else init
    else:
        ref = min(x.min(), init) if n else init
    if np.dtype(dt).kind == "f" and op == "plus":
        assert abs(float(got) - float(ref)) <= 1e-4 * (np.abs(x).sum() + 3) + 1e-6
    else:
        assert got == ref


def test_reduce_deterministic(mgpu, ctx, rng):
    x = rng.standard_normal(3_000_000).astype(np.float32)
    d = mgpu.DeviceArray.from_numpy(x)
    outs = []
    for _ in range(3):
        o = mgpu.DeviceArray(1, np.float32)
        ctx.reduce(d, o)
        ctx.synchronize()
        outs.append(o.numpy()[0].view(np.uint32))
    assert outs[0] == outs[1] == outs[2]


@pytest.mark.slow
@pytest.mark.parametrize("scan_type", ["exc", "inc"])
def test_scan_full_size(mgpu, ctx, oracle, scan_type):
    """2^28 int32 U[0,100): bit-exact against the oracle."""
    n = 1 << 28
    rng = np.random.default_rng(0x6D677075 + 1)
    x = rng.integers(0, 100, n).astype(np.int32)
    got, _ = run_scan(mgpu, ctx, x, scan_type)
    ref = oracle.scan_int(x, exclusive=scan_type == "exc")
    assert np.array_equal(got, ref)


@pytest.mark.slow
def test_scan_f32_full_size(mgpu, ctx, oracle):
    """2^26 float32 N(0,1) inclusive scan against the float64 oracle."""
    n = 1 << 26
    rng = np.random.default_rng(0x6D677075 + 3)
    x = rng.standard_normal(n).astype(np.float32)
    got, _ = run_scan(mgpu, ctx, x, "inc")
    ref, ref_abs = oracle.scan_fp(x, exclusive=False)
    err = np.abs(got.astype(np.float64) - ref)
    bound = F32_REL * ref_abs + F32_ABS
    assert np.all(err <= bound), float(np.max(err / bound))


@pytest.mark.parametrize("dt", [np.int32, np.int64])
@pytest.mark.parametrize("scan_type", ["exc", "inc"])
def test_scan_every_variant_unaligned_and_ragged(mgpu, ctx, oracle, rng, dt, scan_type):
    """Every launch shape, with 16-byte-aligned pointers (bulk-copied tiles)
    and with pointers one element off (tiles read element by element), at
    sizes that end in a ragged tile."""
    import torch
    itemsize = np.dtype(dt).itemsize
    names = ctx.tuning_variants("scan", dt)
    try:
        for var in range(len(names)):
            ctx.tuning_set("scan", dt, 0, -1, var)
            for n in (70_001, 1_000_003):
                x = ints(rng, n, dt, hi=1 << 20)
                ref = oracle.scan_int(x, exclusive=scan_type == "exc")
                for shift in (0, 1):
                    src = mgpu.DeviceArray(n + 1, dt)
                    dst = mgpu.DeviceArray(n + 1, dt)
                    din = mgpu.DeviceArray(n, dt, tensor=src.tensor[shift * itemsize:])
                    dout = mgpu.DeviceArray(n, dt, tensor=dst.tensor[shift * itemsize:])
                    din.tensor[: n * itemsize].copy_(torch.from_numpy(x.view(np.uint8)))
                    red = mgpu.DeviceArray(1, dt)
                    ctx.scan(din, dout, scan_type=scan_type, reduction=red)
                    ctx.synchronize()
                    assert np.array_equal(dout.numpy(), ref), (names[var], n, shift)
                    total = x.astype(np.int64).sum().astype(dt)
                    assert red.numpy()[0] == total, (names[var], n, shift)
    finally:
        ctx.tuning_set("scan", dt, 0, -1, 0)
