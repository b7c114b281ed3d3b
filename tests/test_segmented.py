"""Parity of the batched segmented sort and segmented scan with the host
oracle (per-segment std::stable_sort by radix bits / per-segment scans),
bit-exact for integer work."""
import numpy as np
import pytest

from datagen import keys as gen_keys

pytestmark = pytest.mark.gpu


def lognormal_offsets(rng, num_segments, median=256, sigma=2.0, lo=1, hi=1 << 20):
    lens = np.exp(rng.normal(np.log(median), sigma, num_segments)).round()
    lens = np.clip(lens, lo, hi).astype(np.int64)
    off = np.zeros(num_segments + 1, np.int64)
    np.cumsum(lens, out=off[1:])
    return off


def run_segsort(mgpu, ctx, k, v, off):
    dk = mgpu.DeviceArray.from_numpy(k)
    dv = None if v is None else mgpu.DeviceArray.from_numpy(v)
    do = mgpu.DeviceArray.from_numpy(off)
    ctx.segmented_sort(dk, dv, do)
    ctx.synchronize()
    return dk.numpy(), (None if dv is None else dv.numpy())


def bits(a):
    return a.view(np.uint32 if a.dtype.itemsize == 4 else np.uint64)


# Class limits: 32 (warp), 32 x 21 = 672 and 32 x 13 = 416 (one warp's
# slice for 4- and 8-byte elements), 256 x 21 = 5376 and 256 x 13 = 3328 (one
# CTA); above them onesweep tiles of 7296 (4096) keys, ragged at the end.
# Inside a class the items per thread drop to 3, 7 or 13 when those cover the
# segment: limits 96 / 224 / 416 for a warp, 768 / 1792 / 3328 for a CTA.
@pytest.mark.parametrize("lens", [
    [0], [1], [2], [32], [33], [96], [97], [224], [225], [336], [337], [416], [417], [512],
    [513], [672], [673], [768], [769], [1792], [1793], [2688], [2689], [3328], [3329],
    [4096], [4097], [5376], [5377], [7297], [2 * 7296 + 5], [0, 5, 0, 70, 1, 0],
    [10_000, 1, 3, 4096, 4097, 100_000, 31, 512, 600],
])
@pytest.mark.parametrize("kt", [np.uint32, np.float64])
def test_segsort_classes(mgpu, ctx, oracle, rng, lens, kt):
    off = np.zeros(len(lens) + 1, np.int64)
    np.cumsum(lens, out=off[1:])
    n = int(off[-1])
    k = gen_keys(rng, n, kt, "distinct256")
    v = np.arange(n, dtype=np.uint32)
    gk, gv = run_segsort(mgpu, ctx, k, v, off)
    ok, ov = oracle.segmented_sort(k, v, off, mode="radix")
    assert np.array_equal(bits(gk), bits(ok)) and np.array_equal(gv, ov)


@pytest.mark.parametrize("kt", [np.uint32, np.int32, np.float32, np.uint64, np.int64, np.float64])
@pytest.mark.parametrize("vt", [None, np.uint32, np.uint64])
def test_segsort_types(mgpu, ctx, oracle, rng, kt, vt):
    off = lognormal_offsets(rng, 500, median=200, sigma=1.5, hi=30_000)
    n = int(off[-1])
    k = gen_keys(rng, n, kt)
    v = None if vt is None else np.arange(n).astype(vt)
    gk, gv = run_segsort(mgpu, ctx, k, v, off)
    ok, ov = oracle.segmented_sort(k, v, off, mode="radix")
    assert np.array_equal(bits(gk), bits(ok))
    if vt is not None:
        assert np.array_equal(gv, ov)


def test_segsort_lognormal_batch(mgpu, ctx, oracle):
    """The batched configuration's shape at reduced count: lognormal lengths
    (median 256, sigma 2, clipped to [1, 2^20]) over 5,000 segments."""
    rng = np.random.default_rng(0x6D677075 + 3)
    off = lognormal_offsets(rng, 5000)
    n = int(off[-1])
    k = gen_keys(rng, n, np.uint32)
    v = np.arange(n, dtype=np.uint32)
    gk, gv = run_segsort(mgpu, ctx, k, v, off)
    ok, ov = oracle.segmented_sort(k, v, off, mode="radix")
    assert np.array_equal(gk, ok) and np.array_equal(gv, ov)


def run_segscan(mgpu, ctx, x, off, scan_type, op="plus", init=None):
    d = mgpu.DeviceArray.from_numpy(x)
    o = mgpu.DeviceArray(x.size, x.dtype)
    do = mgpu.DeviceArray.from_numpy(off)
    ctx.segmented_scan(d, o, do, scan_type=scan_type, op=op, init=init)
    ctx.synchronize()
    return o.numpy()


@pytest.mark.parametrize("lens", [[1], [7], [4096], [4097], [1, 1, 1, 1], [0, 3, 0, 0, 9000, 2],
                                  [100_000], [5000] * 40])
@pytest.mark.parametrize("scan_type", ["exc", "inc"])
def test_segscan_shapes(mgpu, ctx, oracle, rng, lens, scan_type):
    off = np.zeros(len(lens) + 1, np.int64)
    np.cumsum(lens, out=off[1:])
    x = rng.integers(-100, 100, int(off[-1])).astype(np.int32)
    got = run_segscan(mgpu, ctx, x, off, scan_type)
    ref = oracle.segmented_scan_int(x, off, exclusive=scan_type == "exc")
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("dt", [np.int32, np.uint32, np.int64, np.uint64])
@pytest.mark.parametrize("op", ["plus", "max", "min"])
@pytest.mark.parametrize("scan_type", ["exc", "inc"])
def test_segscan_ops(mgpu, ctx, oracle, rng, dt, op, scan_type):
    off = lognormal_offsets(rng, 3000, median=100, sigma=2.0, hi=200_000)
    n = int(off[-1])
    x = rng.integers(0, 1000, n).astype(dt)
    info = np.iinfo(dt)
    init = {"plus": 7, "max": info.min, "min": info.max}[op]
    got = run_segscan(mgpu, ctx, x, off, scan_type, op=op, init=init)
    ref = oracle.segmented_scan_int(x, off, exclusive=scan_type == "exc", init=init, op=op)
    assert np.array_equal(got, ref)


@pytest.mark.slow
def test_segsort_full_batch(mgpu, ctx, oracle):
    """100,000 lognormal segments (median 256, sigma 2, clipped [1, 2^20]),
    about 2^27 u32 keys + u32 values: exact against per-segment stable sorts."""
    rng = np.random.default_rng(0x6D677075 + 3)
    off = lognormal_offsets(rng, 100_000)
    n = int(off[-1])
    k = gen_keys(rng, n, np.uint32)
    v = np.arange(n, dtype=np.uint32)
    gk, gv = run_segsort(mgpu, ctx, k, v, off)
    ok, ov = oracle.segmented_sort(k, v, off, mode="radix")
    assert np.array_equal(gk, ok) and np.array_equal(gv, ov)


@pytest.mark.slow
@pytest.mark.parametrize("scan_type", ["inc", "exc"])
def test_segscan_full_batch(mgpu, ctx, oracle, scan_type):
    """The segmented-scan configuration: the 100,000 lognormal segments
    (median 256, sigma 2, clipped [1, 2^20]) over int32 U[0,100) values,
    plus; exact against per-segment scans on the host."""
    rng = np.random.default_rng(0x6D677075 + 2 + 8)     # the benchmark's seed
    off = lognormal_offsets(rng, 100_000)
    n = int(off[-1])
    x = rng.integers(0, 100, n).astype(np.int32)
    got = run_segscan(mgpu, ctx, x, off, scan_type)
    ref = oracle.segmented_scan_int(x, off, exclusive=scan_type == "exc")
    assert np.array_equal(got, ref)
