"""Parity of mgpu_radix_sort (onesweep, sm_103a) with the host oracle.

The oracle is std::stable_sort by radix_permute_t bits (reference:
vk/radix.hxx:195-470, common/cta_radix.hxx:6-64), bit-exact: keys compared as
raw bits (so -0.0/+0.0 and NaN payloads count), values compared exactly.
"""
import numpy as np
import pytest

from datagen import keys as gen_keys
from datagen import wide_keys

pytestmark = pytest.mark.gpu

# Around the one-CTA limits (3072 keys of 8 bytes, 5120 of 4 bytes; the
# one-CTA sort takes 3 items per thread up to 3072 keys) and the onesweep
# tiles (4096 for 8-byte keys or values, 7296 otherwise).
SIZES = [0, 1, 2, 31, 32, 33, 255, 2560, 2561, 3072, 3073, 4095, 4096, 4097, 5120, 5121, 7296,
         7297, 3 * 4096 + 5, 2 * 7296 + 1, 65536 + 7, 300_001]
KEY_TYPES = [np.uint32, np.int32, np.float32, np.uint64, np.int64, np.float64]


def bits(a):
    return a.view(np.uint32 if a.dtype.itemsize == 4 else np.uint64)


def run_sort(mgpu, ctx, k, v):
    dk = mgpu.DeviceArray.from_numpy(k)
    dv = None if v is None else mgpu.DeviceArray.from_numpy(v)
    ctx.radix_sort(dk, dv)
    ctx.synchronize()
    return dk.numpy(), (None if dv is None else dv.numpy())


@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("kt", KEY_TYPES)
def test_radix_sizes(mgpu, ctx, oracle, rng, n, kt):
    k = gen_keys(rng, n, kt)
    v = np.arange(n, dtype=np.uint32)
    gk, gv = run_sort(mgpu, ctx, k, v)
    ok, ov = oracle.radix_sort(k, v)
    assert np.array_equal(bits(gk), bits(ok))
    assert np.array_equal(gv, ov)


@pytest.mark.parametrize("dist", ["uniform", "and2", "distinct256", "equal", "two", "sorted",
                                  "reverse"])
@pytest.mark.parametrize("kt", [np.uint32, np.uint64, np.int32])
def test_radix_distributions(mgpu, ctx, oracle, rng, dist, kt):
    n = 200_003
    k = gen_keys(rng, n, kt, dist)
    v = np.arange(n, dtype=np.uint32)
    gk, gv = run_sort(mgpu, ctx, k, v)
    ok, ov = oracle.radix_sort(k, v)
    assert np.array_equal(bits(gk), bits(ok))
    assert np.array_equal(gv, ov)


@pytest.mark.parametrize("dist", ["distinct256", "equal", "two", "sorted", "reverse"])
@pytest.mark.parametrize("n", [300, 2500, 4000])
@pytest.mark.parametrize("kt", [np.uint32, np.float32, np.uint64])
def test_radix_one_cta_distributions(mgpu, ctx, oracle, rng, dist, n, kt):
    """Sorts that fit one CTA (a merge sort in shared memory) keep equal
    keys in input order."""
    k = gen_keys(rng, n, kt, dist)
    v = np.arange(n, dtype=np.uint32)
    gk, gv = run_sort(mgpu, ctx, k, v)
    ok, ov = oracle.radix_sort(k, v)
    assert np.array_equal(bits(gk), bits(ok))
    assert np.array_equal(gv, ov)


@pytest.mark.parametrize("kt", [np.float32, np.float64])
def test_radix_float_bit_order(mgpu, ctx, oracle, rng, kt):
    """-0.0 before +0.0 and NaNs placed by bit pattern (radix_permute_t)."""
    n = 50_000
    k = gen_keys(rng, n, kt, "fbits")
    v = np.arange(n, dtype=np.uint32)
    gk, gv = run_sort(mgpu, ctx, k, v)
    ok, ov = oracle.radix_sort(k, v)
    assert np.array_equal(bits(gk), bits(ok))
    assert np.array_equal(gv, ov)


@pytest.mark.parametrize("vt", [None, np.uint32, np.uint64])
@pytest.mark.parametrize("kt", [np.uint32, np.float64])
def test_radix_value_widths(mgpu, ctx, oracle, rng, kt, vt):
    n = 100_000
    k = gen_keys(rng, n, kt, "distinct256")
    v = None if vt is None else rng.integers(0, 2 ** 31, n).astype(vt)
    gk, gv = run_sort(mgpu, ctx, k, v)
    ok, ov = oracle.radix_sort(k, v)
    assert np.array_equal(bits(gk), bits(ok))
    if v is not None:
        assert np.array_equal(gv, ov)


def test_radix_two_phase_aux(mgpu, ctx, oracle, rng):
    """Caller-owned aux: a sizing call, then a run with that capacity; a run
    with less capacity is rejected (vk/radix.hxx:288-302 sizing protocol)."""
    import torch
    n = 123_457
    k = gen_keys(rng, n, np.uint32)
    v = np.arange(n, dtype=np.uint32)
    size = ctx.radix_sort_aux_size(np.uint32, np.uint32, n)
    assert size > 0
    aux = torch.empty(size, dtype=torch.uint8, device="cuda")
    dk = mgpu.DeviceArray.from_numpy(k)
    dv = mgpu.DeviceArray.from_numpy(v)
    ctx.radix_sort(dk, dv, aux=(aux.data_ptr(), size))
    ctx.synchronize()
    ok, ov = oracle.radix_sort(k, v)
    assert np.array_equal(dk.numpy(), ok) and np.array_equal(dv.numpy(), ov)
    with pytest.raises(mgpu.MgpuError):
        ctx.radix_sort(dk, dv, aux=(aux.data_ptr(), size - 1))
    # aux that does not start on 16 bytes is rejected before any launch.
    aux2 = torch.empty(size + 16, dtype=torch.uint8, device="cuda")
    with pytest.raises(mgpu.MgpuError):
        ctx.radix_sort(dk, dv, aux=(aux2.data_ptr() + 4, size))
    dsrc = mgpu.DeviceArray.from_numpy(np.arange(1000, dtype=np.int32))
    seg = mgpu.DeviceArray.from_numpy(np.array([0, 400, 1000], dtype=np.int64))
    with pytest.raises(mgpu.MgpuError):
        ctx.segmented_scan(dsrc, dsrc, seg, aux=(aux2.data_ptr() + 8, size))
    ctx.synchronize()


def test_radix_unaligned_pointers(mgpu, ctx, oracle, rng):
    """Buffers that do not start on 16 bytes take the plain-load path."""
    n = 70_001
    k = gen_keys(rng, n + 1, np.uint32)
    v = np.arange(n + 1, dtype=np.uint32)
    dk = mgpu.DeviceArray.from_numpy(k)
    dv = mgpu.DeviceArray.from_numpy(v)
    sub_k = mgpu.DeviceArray(n, np.uint32, tensor=dk.tensor[4:])
    sub_v = mgpu.DeviceArray(n, np.uint32, tensor=dv.tensor[4:])
    ctx.radix_sort(sub_k, sub_v)
    ctx.synchronize()
    ok, ov = oracle.radix_sort(k[1:], v[1:])
    assert np.array_equal(sub_k.numpy(), ok) and np.array_equal(sub_v.numpy(), ov)


def test_radix_reference_kat_shape(mgpu, ctx, oracle):
    """The reference's own known-answer check (examples/vk_radix2/
    vk_radix2.cxx:13-75): 256*32^3 glibc rand() keys, sorted six times in a
    row, equal to std::sort."""
    n = 256 * 32 * 32 * 32
    k = oracle.libc_rand(n, 1)
    dk = mgpu.DeviceArray.from_numpy(k)
    for _ in range(6):
        ctx.radix_sort(dk)
    ctx.synchronize()
    assert np.array_equal(dk.numpy(), np.sort(k))


@pytest.mark.slow
@pytest.mark.parametrize("dist", ["uniform", "and2", "distinct256"])
def test_radix_full_size_properties(mgpu, ctx, dist):
    """2^28 u32 keys + u32 values (the headline workload): the output is the
    unique stable permutation iff keys are sorted, out_keys == in_keys[vals],
    vals is a permutation, and equal keys keep increasing vals."""
    n = 1 << 28
    rng = np.random.default_rng(0x6D677075 + 2)
    k = gen_keys(rng, n, np.uint32, dist)
    v = np.arange(n, dtype=np.uint32)
    dk = mgpu.DeviceArray.from_numpy(k)
    dv = mgpu.DeviceArray.from_numpy(v)
    ctx.radix_sort(dk, dv)
    ctx.synchronize()
    gk, gv = dk.numpy(), dv.numpy()
    assert np.all(gk[1:] >= gk[:-1])
    assert np.array_equal(k[gv], gk)
    seen = np.zeros(n, dtype=bool)
    seen[gv] = True
    assert seen.all()
    eq = gk[1:] == gk[:-1]
    assert np.all(gv[1:][eq] > gv[:-1][eq])


@pytest.mark.slow
@pytest.mark.parametrize("kind", ["u64", "f32bits", "f32normal"])
def test_radix_wide_full_size_exact(mgpu, ctx, oracle, kind):
    """The 2^27-key configurations with int32 values = index: u64 uniform
    64-bit keys, and f32 keys as uniform finite bit patterns and as N(0,1);
    bit-exact against the oracle's parallel stable sort by radix bits."""
    n = 1 << 27
    # The benchmark's generator and seeds (bench.py wl_radix_wide).
    rng = np.random.default_rng(0x6D677075 + 2 + (6 if kind == "u64" else 7))
    k = wide_keys(rng, n, kind)
    v = np.arange(n, dtype=np.int32)
    dk = mgpu.DeviceArray.from_numpy(k)
    dv = mgpu.DeviceArray.from_numpy(v)
    ctx.radix_sort(dk, dv)
    ctx.synchronize()
    gk, gv = dk.numpy(), dv.numpy()
    del dk, dv
    ok, ov = oracle.sort_parallel(k, v, mode="radix")
    assert np.array_equal(bits(gk), bits(ok))
    assert np.array_equal(gv, ov)


def test_radix_orders_with_torch_stream(mgpu, ctx, oracle, rng):
    """Work enqueued by torch on its current stream (an async device copy)
    is ordered before the sort: the context enqueues on the same stream."""
    n = 4_000_037
    k = gen_keys(rng, n, np.uint32)
    v = np.arange(n, dtype=np.uint32)
    src_k, src_v = mgpu.DeviceArray.from_numpy(k), mgpu.DeviceArray.from_numpy(v)
    dk, dv = mgpu.DeviceArray(n, np.uint32), mgpu.DeviceArray(n, np.uint32)
    for _ in range(3):
        dk.copy_from(src_k)          # async on torch's stream
        dv.copy_from(src_v)
        ctx.radix_sort(dk, dv)       # no host synchronisation in between
    ctx.synchronize()
    ok, ov = oracle.radix_sort(k, v)
    assert np.array_equal(dk.numpy(), ok) and np.array_equal(dv.numpy(), ov)
