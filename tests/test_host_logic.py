"""Host-side logic that needs no GPU: the compiled launch-shape lists the
tuner chooses from (read through the C ABI), and the output checks the
benchmark reports, each shown to catch a planted mistake."""
import numpy as np
import pytest

import bench


def test_tuning_variant_lists(mgpu):
    tv = mgpu.tuning_variants
    assert tv("radix", np.uint32) == ["384x19", "256x31", "256x23", "256x16/4b", "128x16/4b"]
    assert tv("radix", np.float64) == ["256x16", "256x12", "384x10", "256x16/4b", "128x16/4b"]
    assert tv("scan", np.int32) == ["256x32b4p", "512x32b2p", "256x16b6p", "256x32b4t"]
    assert tv("scan", np.int64) == ["512x16b2p", "256x16b4p", "256x8b6p", "256x16b4t"]
    assert tv("merge", np.int32) == ["256x15", "256x8", "256x16"]
    assert tv("merge", np.uint64) == ["256x7", "128x8", "256x8"]
    assert tv("mergesort", np.float32) == ["256x15", "256x8", "256x17"]
    assert tv("mergesort", np.int64) == ["256x7", "128x8", "256x8"]
    # The radix lists offer both digit widths, so the autotuner picks one.
    for kt in (np.uint32, np.uint64):
        names = tv("radix", kt)
        assert any(s.endswith("/4b") for s in names) and any("/" not in s for s in names)


def stable_sort_of(keys):
    order = np.argsort(keys, kind="stable")
    return keys[order], order.astype(np.uint32)


def test_stable_sort_checks_pass_the_stable_sort_only():
    rng = np.random.default_rng(7)
    keys = rng.integers(0, 50, 5000).astype(np.uint32)
    gk, gv = stable_sort_of(keys)
    assert all(bench.stable_sort_checks(keys, gk, gv).values())

    # Two equal keys' values swapped: sorted, a permutation, values carry
    # their keys, but not stable.
    i = int(np.flatnonzero(gk[1:] == gk[:-1])[0])
    bad = gv.copy()
    bad[i], bad[i + 1] = bad[i + 1], bad[i]
    c = bench.stable_sort_checks(keys, gk, bad)
    assert c["values_are_a_permutation"] and c["values_carry_their_keys"]
    assert not c["equal_keys_keep_input_order"]

    # One index written twice: no longer a permutation.
    bad = gv.copy()
    bad[10] = bad[11]
    assert not bench.stable_sort_checks(keys, gk, bad)["values_are_a_permutation"]

    # Keys out of order.
    bad_k = gk.copy()
    bad_k[0], bad_k[-1] = bad_k[-1], bad_k[0]
    assert not bench.stable_sort_checks(keys, bad_k, gv)["keys_ascend"]

    # An index out of range is reported, not raised.
    bad = gv.copy()
    bad[0] = keys.size
    c = bench.stable_sort_checks(keys, gk, bad)
    assert not c["values_are_a_permutation"] and not c["values_carry_their_keys"]


def test_segmented_sort_checks_catch_a_value_leaving_its_segment():
    rng = np.random.default_rng(8)
    lens = np.array([0, 5, 300, 1, 64, 1000])
    off = np.zeros(lens.size + 1, np.int64)
    np.cumsum(lens, out=off[1:])
    keys = rng.integers(0, 20, int(off[-1])).astype(np.uint32)
    gk, gv = keys.copy(), np.arange(keys.size, dtype=np.uint32)
    for s in range(lens.size):
        b, e = off[s], off[s + 1]
        order = np.argsort(keys[b:e], kind="stable")
        gk[b:e] = keys[b:e][order]
        gv[b:e] = (b + order).astype(np.uint32)
    assert all(bench.segmented_sort_checks(keys, off, gk, gv).values())

    # Sorting the whole array instead of each segment: every key ascends
    # globally, but values leave their segments.
    wk, wv = stable_sort_of(keys)
    c = bench.segmented_sort_checks(keys, off, wk, wv)
    assert c["values_are_a_permutation"] and not c["values_stay_in_their_segment"]


@pytest.mark.parametrize("n", [1 << 10, 1 << 20])
def test_make_input_is_seeded(n):
    a_k, a_v = bench.make_input(n)
    b_k, b_v = bench.make_input(n)
    assert np.array_equal(a_k, b_k) and np.array_equal(a_v, b_v)
    assert np.array_equal(a_v, np.arange(n, dtype=a_v.dtype))
