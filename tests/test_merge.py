"""Parity of mgpu_merge / mgpu_mergesort / mgpu_mergesort_indices with the
host oracle (std::merge / std::stable_sort), bit-exact.  Ties: merge takes A
first and mergesort is stable (reference: merge_path bounds_lower,
common/cta_merge.hxx:23-25; odd_even_sort strict swaps,
common/sort_networks.hxx:17,30)."""
import numpy as np
import pytest

from datagen import keys as gen_keys

pytestmark = pytest.mark.gpu

KEY_TYPES = [np.int32, np.uint32, np.float32, np.int64, np.uint64, np.float64]


def dev(mgpu, x):
    return mgpu.DeviceArray.from_numpy(x)


def dup_keys(rng, n, kt, hi=1000):
    kt = np.dtype(kt)
    if kt.kind == "f":
        return (rng.integers(0, hi, n) / 4).astype(kt)
    return rng.integers(0, hi, n).astype(kt)


def run_merge(mgpu, ctx, a, av, b, bv, comp):
    da, db = dev(mgpu, a), dev(mgpu, b)
    dav = None if av is None else dev(mgpu, av)
    dbv = None if bv is None else dev(mgpu, bv)
    dc = mgpu.DeviceArray(a.size + b.size, a.dtype)
    dcv = None if av is None else mgpu.DeviceArray(a.size + b.size, av.dtype)
    ctx.merge(da, dav, db, dbv, dc, dcv, comp=comp)
    ctx.synchronize()
    return dc.numpy(), (None if dcv is None else dcv.numpy())


@pytest.mark.parametrize("an,bn", [(0, 0), (0, 1), (1, 0), (1, 1), (17, 4096), (4096, 4096),
                                   (4095, 1), (10_000, 3), (100_003, 99_991), (300_000, 7)])
@pytest.mark.parametrize("kt", [np.int32, np.float64])
def test_merge_sizes(mgpu, ctx, oracle, rng, an, bn, kt):
    a = np.sort(dup_keys(rng, an, kt))
    b = np.sort(dup_keys(rng, bn, kt))
    av = np.arange(an, dtype=np.int32)
    bv = np.arange(bn, dtype=np.int32) + 10_000_000
    gk, gv = run_merge(mgpu, ctx, a, av, b, bv, "less")
    ok, ov = oracle.merge(a, av, b, bv)
    assert np.array_equal(gk, ok) and np.array_equal(gv, ov)


@pytest.mark.parametrize("kt", KEY_TYPES)
@pytest.mark.parametrize("vt", [None, np.uint32, np.uint64])
@pytest.mark.parametrize("comp", ["less", "greater"])
def test_merge_types(mgpu, ctx, oracle, rng, kt, vt, comp):
    an, bn = 70_001, 50_023
    a = np.sort(dup_keys(rng, an, kt, hi=300))
    b = np.sort(dup_keys(rng, bn, kt, hi=300))
    if comp == "greater":
        a, b = a[::-1].copy(), b[::-1].copy()
    av = None if vt is None else np.arange(an).astype(vt)
    bv = None if vt is None else (np.arange(bn) + 1_000_000).astype(vt)
    gk, gv = run_merge(mgpu, ctx, a, av, b, bv, comp)
    ok, ov = oracle.merge(a, av, b, bv, mode=comp)
    assert np.array_equal(gk, ok)
    if vt is not None:
        assert np.array_equal(gv, ov)


def test_merge_unaligned_inputs(mgpu, ctx, oracle, rng):
    """Sub-buffers that start off a 16-byte boundary use plain loads."""
    a = np.sort(dup_keys(rng, 40_001, np.int32))
    b = np.sort(dup_keys(rng, 30_002, np.int32))
    da_full = dev(mgpu, np.concatenate([[0], a]).astype(np.int32))
    db_full = dev(mgpu, np.concatenate([[0], b]).astype(np.int32))
    da = mgpu.DeviceArray(a.size, np.int32, tensor=da_full.tensor[4:])
    db = mgpu.DeviceArray(b.size, np.int32, tensor=db_full.tensor[4:])
    dc = mgpu.DeviceArray(a.size + b.size, np.int32)
    ctx.merge(da, None, db, None, dc, None)
    ctx.synchronize()
    ok, _ = oracle.merge(a, None, b, None)
    assert np.array_equal(dc.numpy(), ok)


def test_merge_all_equal_keys_take_a_first(mgpu, ctx, oracle):
    a = np.full(10_000, 5, np.int32)
    b = np.full(12_345, 5, np.int32)
    av = np.arange(a.size, dtype=np.int32)
    bv = -1 - np.arange(b.size, dtype=np.int32)
    gk, gv = run_merge(mgpu, ctx, a, av, b, bv, "less")
    assert np.array_equal(gv[: a.size], av) and np.array_equal(gv[a.size:], bv)


def run_mergesort(mgpu, ctx, k, v, comp):
    dk = dev(mgpu, k)
    dv = None if v is None else dev(mgpu, v)
    ctx.mergesort(dk, dv, comp=comp)
    ctx.synchronize()
    return dk.numpy(), (None if dv is None else dv.numpy())


# 3840 = one 256 x 15 tile (u32 keys + u32 values): 2^20 keys take 274 tiles
# and nine passes.
@pytest.mark.parametrize("n", [0, 1, 2, 15, 16, 17, 255, 3839, 3840, 3841, 4095, 4096, 4097,
                               7680, 7681, 8192, 8193, 3 * 4096 + 11, 100_000, 1 << 20,
                               (1 << 20) + 3840 * 15])
def test_mergesort_sizes(mgpu, ctx, oracle, rng, n):
    k = dup_keys(rng, n, np.uint32)
    v = np.arange(n, dtype=np.uint32)
    gk, gv = run_mergesort(mgpu, ctx, k, v, "less")
    ok, ov = oracle.sort(k, v, mode="less")
    assert np.array_equal(gk, ok) and np.array_equal(gv, ov)


@pytest.mark.parametrize("kt", KEY_TYPES)
@pytest.mark.parametrize("vt", [None, np.uint32, np.uint64])
@pytest.mark.parametrize("comp", ["less", "greater"])
def test_mergesort_types(mgpu, ctx, oracle, rng, kt, vt, comp):
    n = 150_001
    k = dup_keys(rng, n, kt, hi=500)
    v = None if vt is None else np.arange(n).astype(vt)
    gk, gv = run_mergesort(mgpu, ctx, k, v, comp)
    ok, ov = oracle.sort(k, v, mode=comp)
    assert np.array_equal(gk, ok)
    if vt is not None:
        assert np.array_equal(gv, ov)


@pytest.mark.parametrize("dist", ["equal", "two", "sorted", "reverse", "uniform"])
def test_mergesort_distributions(mgpu, ctx, oracle, rng, dist):
    n = 200_001
    k = gen_keys(rng, n, np.int32, dist)
    v = np.arange(n, dtype=np.uint32)
    gk, gv = run_mergesort(mgpu, ctx, k, v, "less")
    ok, ov = oracle.sort(k, v, mode="less")
    assert np.array_equal(gk, ok) and np.array_equal(gv, ov)


@pytest.mark.parametrize("n", [3000, 100_003, 1 << 20])
def test_mergesorts_chained_without_a_sync(mgpu, ctx, oracle, rng, n):
    """The blocksort and merge passes start as programmatic dependents of the
    kernel before them: back-to-back sorts of one array on one stream (a
    radix sort, then two mergesorts) must each see the previous result."""
    k = dup_keys(rng, n, np.uint32, hi=700)
    v = np.arange(n, dtype=np.uint32)
    dk, dv = dev(mgpu, k), dev(mgpu, v)
    ctx.radix_sort(dk, dv)
    ctx.mergesort(dk, dv, comp="greater")
    ctx.mergesort(dk, dv, comp="less")
    ctx.synchronize()
    k1, v1 = oracle.radix_sort(k, v)
    k2, v2 = oracle.sort(k1, v1, mode="greater")
    k3, v3 = oracle.sort(k2, v2, mode="less")
    assert np.array_equal(dk.numpy(), k3) and np.array_equal(dv.numpy(), v3)


@pytest.mark.parametrize("n", [1, 10_000, 1 << 20])
def test_mergesort_indices(mgpu, ctx, oracle, rng, n):
    """vk::mergesort_indices, checked like examples/gl_sort/gl_sort.cxx:18-27:
    gathering the input by the indices gives the sorted keys."""
    k = (rng.integers(0, 10_000, n)).astype(np.float32)
    dk = dev(mgpu, k)
    di = mgpu.DeviceArray(n, np.int32)
    ctx.mergesort_indices(dk, di)
    ctx.synchronize()
    gk, gi = dk.numpy(), di.numpy()
    assert np.all(gk[1:] >= gk[:-1])
    assert np.array_equal(k[gi], gk)
    ok, oi = oracle.sort(k, np.arange(n, dtype=np.int32), mode="less")
    assert np.array_equal(gk, ok) and np.array_equal(gi, oi)


@pytest.mark.slow
def test_merge_full_size(mgpu, ctx, oracle):
    """2^26 + 2^26 int32 keys drawn from [0, 2^24) (about 25% duplicates),
    int32 values; exact against std::merge."""
    rng = np.random.default_rng(0x6D677075 + 1)
    n = 1 << 26
    a = np.sort(rng.integers(0, 1 << 24, n).astype(np.int32))
    b = np.sort(rng.integers(0, 1 << 24, n).astype(np.int32))
    av = np.arange(n, dtype=np.int32)
    bv = (np.arange(n) + n).astype(np.int32)
    gk, gv = run_merge(mgpu, ctx, a, av, b, bv, "less")
    ok, ov = oracle.merge(a, av, b, bv)
    assert np.array_equal(gk, ok) and np.array_equal(gv, ov)
