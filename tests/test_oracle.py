"""CPU tests of the oracle (test infrastructure).

The std:: oracle (oracle/oracle.cpp) is pinned against the restatement of the
reference's own tile algorithms (oracle/ref_emulation.cpp) and against the
known-answer checks in the reference's examples:
  * examples/vk_radix2/vk_radix2.cxx:13-75  (u32 radix sort == std::sort)
  * examples/gl_sort/gl_sort.cxx:10-43       (keys+indices: sorted, inverse)
  * examples/vk_scan/vk_scan.cxx:13-61       (exclusive scan of i -> i(i-1)/2)
"""
import numpy as np
import pytest


def test_kat_vk_radix2(oracle):
    # 256 * 32^3 glibc rand() keys (default seed), nt=256, vt=1, 8-bit digits,
    # sorted six times in a row; each result equals std::sort.
    n = 256 * 32 * 32 * 32
    k = oracle.libc_rand(n, 1)
    ref = np.sort(k)
    out, _ = oracle.emu_radix_sort(k, None, nt=256, vt=1, num_bits=8)
    assert np.array_equal(out, ref)
    out2, _ = oracle.emu_radix_sort(out, None, nt=256, vt=1, num_bits=8)
    assert np.array_equal(out2, ref)
    o, _ = oracle.radix_sort(k)
    assert np.array_equal(o, ref)


def test_kat_gl_sort(oracle):
    # 10,000 floats rand() % 10000, mergesort keys + indices at nt=128, vt=7:
    # gathering the input by the indices reproduces the sorted keys.
    raw = oracle.libc_rand(10000, 1)
    data = (raw % 10000).astype(np.float32)
    keys, idx = oracle.emu_mergesort(data, None, nt=128, vt=7, sort_indices=True)
    assert np.all(keys[1:] >= keys[:-1])
    assert np.array_equal(data[idx], keys)
    ok, ov = oracle.sort(data, np.arange(data.size, dtype=np.int32))
    assert np.array_equal(ok, keys) and np.array_equal(ov, idx)


def test_kat_vk_scan(oracle):
    n = 10000
    x = np.arange(n, dtype=np.int32)
    expect = (np.arange(n, dtype=np.int64) * (np.arange(n, dtype=np.int64) - 1) // 2).astype(np.int32)
    assert np.array_equal(oracle.emu_scan_exc_i32(x), expect)
    assert np.array_equal(oracle.scan_int(x, exclusive=True), expect)


@pytest.mark.parametrize("n", [0, 1, 2, 31, 895, 896, 897, 5000, 20011])
@pytest.mark.parametrize("comp", ["less", "greater"])
def test_mergesort_emulation_matches_stable_sort(oracle, rng, n, comp):
    k = rng.integers(0, 50, n).astype(np.int32)
    v = np.arange(n, dtype=np.int32)
    ek, ev = oracle.emu_mergesort(k, v, comp=comp)
    ok, ov = oracle.sort(k, v, mode=comp)
    assert np.array_equal(ek, ok) and np.array_equal(ev, ov)


@pytest.mark.parametrize("an,bn", [(0, 0), (1, 0), (0, 9), (700, 3000), (4000, 4001)])
def test_merge_emulation_matches_std_merge(oracle, rng, an, bn):
    a = np.sort(rng.integers(0, 40, an)).astype(np.uint32)
    b = np.sort(rng.integers(0, 40, bn)).astype(np.uint32)
    av = np.arange(an, dtype=np.int32)
    bv = np.arange(bn, dtype=np.int32) + 1_000_000
    ek, ev = oracle.emu_merge(a, av, b, bv)
    ok, ov = oracle.merge(a, av, b, bv)
    assert np.array_equal(ek, ok) and np.array_equal(ev, ov)


@pytest.mark.parametrize("n", [1, 100, 896, 7168, 7169, 60000, 200000])
def test_scan_emulation_matches_exclusive_scan(oracle, rng, n):
    x = rng.integers(-1000, 1000, n).astype(np.int32)
    assert np.array_equal(oracle.emu_scan_exc_i32(x), oracle.scan_int(x, exclusive=True))


def test_scan_wraps_like_32bit_adds(oracle):
    x = np.full(1000, 2 ** 30, dtype=np.int32)
    out = oracle.scan_int(x, exclusive=False)
    expect = (np.cumsum(x.astype(np.int64)) & 0xFFFFFFFF).astype(np.uint32).view(np.int32)
    assert np.array_equal(out, expect)


@pytest.mark.parametrize("bits,nt,vt", [(4, 128, 15), (8, 256, 16), (8, 256, 1)])
@pytest.mark.parametrize("kt", [np.uint32, np.int32, np.float32])
def test_radix_emulation_matches_bit_order(oracle, rng, bits, nt, vt, kt):
    for n in [1, 1000, 4096, 30001]:
        if kt == np.float32:
            k = (rng.standard_normal(n) * 100).astype(kt)
            k[: min(n, 4)] = np.array([0.0, -0.0, 3.0, -3.0], kt)[: min(n, 4)]
        else:
            k = rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32).view(kt)
        v = np.arange(n, dtype=np.int32)
        ek, ev = oracle.emu_radix_sort(k, v, nt=nt, vt=vt, num_bits=bits)
        ok, ov = oracle.radix_sort(k, v)
        assert np.array_equal(ek.view(np.uint32), ok.view(np.uint32))
        assert np.array_equal(ev, ov)


def test_radix_bits_order(oracle):
    f = np.array([-np.inf, -1.0, -0.0, 0.0, 1e-45, 1.0, np.inf], np.float32)
    b = oracle.to_radix_bits(f)
    assert np.all(b[1:] > b[:-1])
    i = np.array([-2 ** 31, -1, 0, 1, 2 ** 31 - 1], np.int32)
    assert np.all(np.diff(oracle.to_radix_bits(i).astype(np.int64)) > 0)


def test_parallel_sort_equals_serial(oracle, rng):
    k = rng.integers(0, 1000, 100_003).astype(np.uint32)
    v = np.arange(k.size, dtype=np.uint32)
    a = oracle.sort(k, v, mode="radix")
    b = oracle.sort_parallel(k, v, mode="radix", threads=7)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_segmented_oracles(oracle, rng):
    off = np.array([0, 0, 5, 6, 100, 100, 357], np.int64)
    k = rng.integers(0, 20, 357).astype(np.uint32)
    v = np.arange(357, dtype=np.uint32)
    sk, sv = oracle.segmented_sort(k, v, off)
    for s in range(off.size - 1):
        b, e = off[s], off[s + 1]
        rk, rv = oracle.sort(k[b:e], v[b:e], mode="radix")
        assert np.array_equal(sk[b:e], rk) and np.array_equal(sv[b:e], rv)
    x = rng.integers(0, 100, 357).astype(np.int32)
    sc = oracle.segmented_scan_int(x, off, exclusive=False)
    for s in range(off.size - 1):
        b, e = off[s], off[s + 1]
        assert np.array_equal(sc[b:e], np.cumsum(x[b:e]).astype(np.int32))
