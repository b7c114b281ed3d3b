"""torch.ops.mgpu.* (mgpu_gb300.torch_ops): registration and argument checks
on the CPU; results against the host oracle and numpy on the GPU, with the
work enqueued on a non-default torch stream."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _ops(mgpu):
    import mgpu_gb300.torch_ops  # noqa: F401  (registers the operators)
    return torch.ops.mgpu


def test_operators_registered(mgpu):
    ops = _ops(mgpu)
    for name in ("radix_sort_", "sort_", "merge", "merge_keys", "scan", "segmented_sort_",
                 "segmented_scan"):
        assert hasattr(ops, name), name
    schema = str(ops.radix_sort_.default._schema)
    assert "!) keys" in schema and "!)? values" in schema     # both mutated in place


def test_cpu_tensors_are_rejected(mgpu):
    ops = _ops(mgpu)
    with pytest.raises(ValueError, match="CUDA tensor"):
        ops.radix_sort_(torch.arange(10, dtype=torch.int32), None)
    with pytest.raises(ValueError, match="CUDA tensor"):
        ops.scan(torch.arange(10, dtype=torch.int64))


def _u32(t):
    return t.cpu().view(torch.int32).numpy().view(np.uint32)


@pytest.mark.gpu
def test_radix_sort_kv_on_side_stream(mgpu, oracle, rng):
    ops = _ops(mgpu)
    n = 300_001
    k = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    v = np.arange(n, dtype=np.int32)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        dk = torch.from_numpy(k.view(np.int32)).cuda().view(torch.uint32)
        dv = torch.from_numpy(v).cuda()
        ops.radix_sort_(dk, dv)
    s.synchronize()
    ok, ov = oracle.radix_sort(k, v.view(np.uint32))
    assert np.array_equal(_u32(dk), ok) and np.array_equal(dv.cpu().numpy().view(np.uint32), ov)


@pytest.mark.gpu
def test_radix_sort_float_bits_and_sort_descending(mgpu, rng):
    ops = _ops(mgpu)
    x = rng.standard_normal(100_000).astype(np.float32)
    d = torch.from_numpy(x).cuda()
    ops.radix_sort_(d, None)
    assert np.array_equal(d.cpu().numpy(), np.sort(x, kind="stable"))
    keys = rng.integers(0, 50, 70_000).astype(np.float64)
    dk = torch.from_numpy(keys).cuda()
    dv = torch.arange(keys.size, dtype=torch.int64, device="cuda")
    ops.sort_(dk, dv, descending=True)
    order = np.argsort(-keys, kind="stable")
    assert np.array_equal(dk.cpu().numpy(), keys[order])
    assert np.array_equal(dv.cpu().numpy(), order)


@pytest.mark.gpu
def test_merge_and_merge_keys(mgpu, rng):
    ops = _ops(mgpu)
    a = np.sort(rng.integers(0, 1000, 40_000)).astype(np.int32)
    b = np.sort(rng.integers(0, 1000, 25_000)).astype(np.int32)
    av = np.arange(a.size, dtype=np.int32)
    bv = np.arange(b.size, dtype=np.int32) + a.size
    ck, cv = ops.merge(*(torch.from_numpy(t).cuda() for t in (a, av, b, bv)))
    keys = np.concatenate([a, b])
    order = np.argsort(keys, kind="stable")       # ties: A first
    assert np.array_equal(ck.cpu().numpy(), keys[order])
    assert np.array_equal(cv.cpu().numpy(), np.concatenate([av, bv])[order])
    ck2 = ops.merge_keys(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda())
    assert np.array_equal(ck2.cpu().numpy(), keys[order])


@pytest.mark.gpu
def test_scan_int32_wraps(mgpu, rng):
    ops = _ops(mgpu)
    x = rng.integers(0, 100, 5_000_000).astype(np.int32)
    d = torch.from_numpy(x).cuda()
    inc = ops.scan(d, inclusive=True).cpu().numpy()
    exc = ops.scan(d).cpu().numpy()
    ref = np.cumsum(x.astype(np.uint32), dtype=np.uint32).view(np.int32)
    assert np.array_equal(inc, ref)
    assert exc[0] == 0 and np.array_equal(exc[1:], ref[:-1])
    mx = ops.scan(d, inclusive=True, op="max").cpu().numpy()
    assert np.array_equal(mx, np.maximum.accumulate(x))


@pytest.mark.gpu
def test_segmented_sort_and_scan(mgpu, oracle, rng):
    ops = _ops(mgpu)
    lens = np.clip(np.exp(rng.normal(np.log(200), 1.5, 2000)).round(), 1, 60_000).astype(np.int64)
    off = np.zeros(lens.size + 1, np.int64)
    np.cumsum(lens, out=off[1:])
    n = int(off[-1])
    k = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    v = np.arange(n, dtype=np.uint32)
    dk = torch.from_numpy(k.view(np.int32)).cuda().view(torch.uint32)
    dv = torch.from_numpy(v.view(np.int32)).cuda()
    do = torch.from_numpy(off).cuda()
    ops.segmented_sort_(dk, dv, do)
    ok, ov = oracle.segmented_sort(k, v, off, mode="radix")
    assert np.array_equal(_u32(dk), ok) and np.array_equal(dv.cpu().numpy().view(np.uint32), ov)
    x = rng.integers(-50, 50, n).astype(np.int32)
    got = ops.segmented_scan(torch.from_numpy(x).cuda(), do, inclusive=True).cpu().numpy()
    assert np.array_equal(got, oracle.segmented_scan_int(x, off, exclusive=False))
    mgpu.torch_ops.synchronize()
