"""The launch-shape tuning table and the autotuner: every compiled variant
gives the oracle's result, the autotuner records a variant for the size
bucket, and tables round-trip through their text file."""
import numpy as np
import pytest

from datagen import keys as gen_keys

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kt", [np.uint32, np.uint64])
def test_every_radix_variant_is_exact(mgpu, ctx, oracle, rng, kt):
    names = ctx.tuning_variants("radix", kt)
    assert len(names) >= 2
    n = 300_017
    k = gen_keys(rng, n, kt)
    v = np.arange(n, dtype=np.uint32)
    ok, ov = oracle.radix_sort(k, v)
    try:
        for var in range(len(names)):
            ctx.tuning_set("radix", kt, 4, -1, var)
            assert ctx.tuning_get("radix", kt, 4, n) == var
            dk, dv = mgpu.DeviceArray.from_numpy(k), mgpu.DeviceArray.from_numpy(v)
            ctx.radix_sort(dk, dv)
            ctx.synchronize()
            assert np.array_equal(dk.numpy(), ok) and np.array_equal(dv.numpy(), ov), names[var]
    finally:
        ctx.tuning_set("radix", kt, 4, -1, 0)


@pytest.mark.parametrize("prim", ["scan", "merge", "mergesort"])
def test_every_variant_other_primitives(mgpu, ctx, oracle, rng, prim):
    n = 200_003
    names = ctx.tuning_variants(prim, np.int32)
    try:
        for var in range(len(names)):
            ctx.tuning_set(prim, np.int32, 0 if prim == "scan" else 4, -1, var)
            x = rng.integers(0, 1000, n).astype(np.int32)
            if prim == "scan":
                d, o = mgpu.DeviceArray.from_numpy(x), mgpu.DeviceArray(n, np.int32)
                ctx.scan(d, o, scan_type="inc")
                ctx.synchronize()
                assert np.array_equal(o.numpy(), oracle.scan_int(x, exclusive=False))
            elif prim == "merge":
                a, b = np.sort(x[: n // 2]), np.sort(x[n // 2:])
                av = np.arange(a.size, dtype=np.uint32)
                bv = np.arange(b.size, dtype=np.uint32) + 10 ** 6
                dc, dcv = mgpu.DeviceArray(n, np.int32), mgpu.DeviceArray(n, np.uint32)
                ctx.merge(mgpu.DeviceArray.from_numpy(a), mgpu.DeviceArray.from_numpy(av),
                          mgpu.DeviceArray.from_numpy(b), mgpu.DeviceArray.from_numpy(bv), dc, dcv)
                ctx.synchronize()
                ok, ov = oracle.merge(a, av, b, bv)
                assert np.array_equal(dc.numpy(), ok) and np.array_equal(dcv.numpy(), ov)
            else:
                v = np.arange(n, dtype=np.uint32)
                dk, dv = mgpu.DeviceArray.from_numpy(x), mgpu.DeviceArray.from_numpy(v)
                ctx.mergesort(dk, dv)
                ctx.synchronize()
                ok, ov = oracle.sort(x, v)
                assert np.array_equal(dk.numpy(), ok) and np.array_equal(dv.numpy(), ov)
    finally:
        ctx.tuning_set(prim, np.int32, 0 if prim == "scan" else 4, -1, 0)


def test_autotune_records_and_round_trips(mgpu, tmp_path):
    c = mgpu.Context(0)
    best, ms = c.autotune("radix", np.uint32, 4, 1 << 22, reps=2)
    assert 0 <= best < len(c.tuning_variants("radix", np.uint32)) and ms > 0
    assert c.tuning_get("radix", np.uint32, 4, 1 << 22) == best
    path = str(tmp_path / "tune.txt")
    c.tuning_save(path)
    c2 = mgpu.Context(0)
    c2.tuning_load(path)
    assert c2.tuning_get("radix", np.uint32, 4, 1 << 22) == best
    b2, _ = c.autotune("scan", np.float32, 0, 1 << 20, reps=2)
    assert c.tuning_get("scan", np.float32, 0, 1 << 20) == b2
    c.close()
    c2.close()


def test_tuning_load_rejects_a_bad_file_whole(mgpu, tmp_path):
    """A table naming a variant that is not compiled (or a bad bucket) is
    refused and leaves the context's table as it was."""
    c = mgpu.Context(0)
    try:
        c.tuning_set("radix", np.uint32, 4, 20, 2)
        good = tmp_path / "good.txt"
        good.write_text("# comment\n0 1 4 22 1\n")
        c.tuning_load(str(good))
        assert c.tuning_get("radix", np.uint32, 4, 1 << 22) == 1
        for body in ("0 1 4 23 1\n0 1 4 24 9\n", "0 1 4 70 1\n", "3 1 4 -1 -1\n"):
            bad = tmp_path / "bad.txt"
            bad.write_text(body)
            with pytest.raises(mgpu.MgpuError):
                c.tuning_load(str(bad))
            assert c.tuning_get("radix", np.uint32, 4, 1 << 23) == 0   # nothing taken
        assert c.tuning_get("radix", np.uint32, 4, 1 << 20) == 2
        with pytest.raises(mgpu.MgpuError):
            c.tuning_load(str(tmp_path / "missing.txt"))
    finally:
        c.close()


@pytest.mark.parametrize("kt", [np.uint32, np.int32, np.float32, np.uint64, np.float64])
@pytest.mark.parametrize("vb", [0, 4, 8])
def test_4bit_digit_variants_are_exact(mgpu, ctx, oracle, rng, kt, vb):
    """The 4-bit-digit passes (the reference's default digit width) give the
    same permutation as the oracle, for every key type and value width, on
    a ragged size and on one below a tile."""
    names = ctx.tuning_variants("radix", kt)
    four = [i for i, nm in enumerate(names) if nm.endswith("/4b")]
    assert four and len(four) < len(names)          # both digit widths are variants
    vdt = {0: None, 4: np.uint32, 8: np.uint64}[vb]
    try:
        for n in (300_017, 9_001):
            k = gen_keys(rng, n, kt)
            v = None if vdt is None else np.arange(n, dtype=vdt)
            ok, ov = oracle.radix_sort(k, v)
            for var in four:
                ctx.tuning_set("radix", kt, vb, -1, var)
                dk = mgpu.DeviceArray.from_numpy(k)
                dv = None if v is None else mgpu.DeviceArray.from_numpy(v)
                ctx.radix_sort(dk, dv)
                ctx.synchronize()
                assert np.array_equal(dk.numpy().view(np.uint8), ok.view(np.uint8)), names[var]
                if v is not None:
                    assert np.array_equal(dv.numpy(), ov), names[var]
    finally:
        ctx.tuning_set("radix", kt, vb, -1, 0)


def test_autotune_chooses_the_digit_width(mgpu):
    """The autotuner times both digit widths and records the fastest variant
    per size bucket; each chosen variant's name states its digit width."""
    c = mgpu.Context(0)
    names = c.tuning_variants("radix", np.uint32)
    widths = {4 if nm.endswith("/4b") else 8 for nm in names}
    assert widths == {4, 8}
    chosen = {}
    for n in (1 << 16, 1 << 20, 1 << 24):
        best, ms = c.autotune("radix", np.uint32, 4, n, reps=2)
        assert ms > 0 and c.tuning_get("radix", np.uint32, 4, n) == best
        chosen[n] = (names[best], 4 if names[best].endswith("/4b") else 8)
    print("autotuned radix variants (size: name, digit bits):", chosen)
    c.close()
