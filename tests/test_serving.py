"""The serving loop (mgpu_server_*): requests admitted under an HBM budget and
run concurrently on several streams give the same bytes as the same request
run alone, and as the oracle; the budget is enforced at submission and at
admission; drain and the latency record behave."""
import numpy as np
import pytest

from datagen import keys as gen_keys

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def server_cls(mgpu):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return mgpu.Server


def make_requests(rng, n_req, max_log2=18):
    """A seeded mix of sort / merge / scan requests with sizes log-uniform in
    [2^4, 2^max_log2] and key types u32 / u64 / f32 / i32 / f64."""
    reqs = []
    for i in range(n_req):
        n = int(2 ** rng.uniform(4, max_log2))
        kind = ["sort", "sort", "merge", "scan"][i % 4]
        kt = [np.uint32, np.uint64, np.float32, np.int32, np.float64][rng.integers(0, 5)]
        if kind == "sort":
            vt = [None, np.uint32, np.uint64][rng.integers(0, 3)]
            k = gen_keys(rng, n, kt)
            v = None if vt is None else rng.integers(0, 2 ** 31, n).astype(vt)
            reqs.append(("sort", k, v))
        elif kind == "merge":
            nb = int(2 ** rng.uniform(0, max_log2))
            a = np.sort(gen_keys(rng, n, kt))
            b = np.sort(gen_keys(rng, nb, kt))
            av = np.arange(n, dtype=np.int32)
            bv = np.arange(nb, dtype=np.int32) + (1 << 30)
            reqs.append(("merge", a, av, b, bv))
        else:
            st = ["exc", "inc"][rng.integers(0, 2)]
            it = [np.int32, np.uint32, np.int64, np.uint64][rng.integers(0, 4)]
            x = rng.integers(0, 1 << 20, n).astype(it)
            reqs.append(("scan", x, st))
    return reqs


def submit(srv, r):
    """Submits one request; returns (id, outputs)."""
    if r[0] == "sort":
        _, k, v = r
        ok = np.empty_like(k)
        ov = None if v is None else np.empty_like(v)
        return srv.submit_sort(k, v, ok, ov), (ok, ov)
    if r[0] == "merge":
        _, a, av, b, bv = r
        ok = np.empty(a.size + b.size, a.dtype)
        ov = np.empty(a.size + b.size, av.dtype)
        return srv.submit_merge(a, av, b, bv, ok, ov), (ok, ov)
    _, x, st = r
    out = np.empty_like(x)
    return srv.submit_scan(x, out, scan_type=st), (out, None)


def expected(oracle, r):
    if r[0] == "sort":
        return oracle.radix_sort(r[1], r[2])
    if r[0] == "merge":
        return oracle.merge(r[1], r[2], r[3], r[4])
    return oracle.scan_int(r[1], exclusive=r[2] == "exc"), None


def same(x, y):
    if x is None or y is None:
        return x is None and y is None
    return np.array_equal(x.view(np.uint8), y.view(np.uint8))


def test_mixed_equals_alone_and_oracle(server_cls, oracle, rng):
    reqs = make_requests(rng, 48)
    # Each request alone: one slot, waited before the next is submitted.
    alone = []
    srv = server_cls(budget_bytes=1 << 30, num_slots=1)
    for r in reqs:
        rid, outs = submit(srv, r)
        srv.wait(rid)
        alone.append(outs)
    srv.close()
    # All at once: four slots, a budget that admits only a few at a time.
    srv = server_cls(budget_bytes=24 << 20, num_slots=4)
    pending = [submit(srv, r) for r in reqs]
    for rid, _ in pending:
        srv.wait(rid)
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert st["peak_bytes"] <= 24 << 20
    for r, a, (_, m) in zip(reqs, alone, pending):
        assert same(a[0], m[0]) and same(a[1], m[1]), r[0]
        ek, ev = expected(oracle, r)
        assert same(ek, m[0]) and same(ev, m[1]), r[0]


def test_budget_rejects_oversized(server_cls, mgpu):
    srv = server_cls(budget_bytes=1 << 20, num_slots=2)
    k = np.zeros(1 << 20, np.uint32)
    with pytest.raises(mgpu.MgpuError) as e:
        srv.submit_sort(k, k.copy(), np.empty_like(k), np.empty_like(k))
    assert e.value.status == 6
    # A request that fits is still served.
    small = np.arange(1000, 0, -1, dtype=np.uint32)
    out = np.empty_like(small)
    srv.wait(srv.submit_sort(small, None, out, None))
    assert np.array_equal(out, np.sort(small))
    srv.close()


def test_budget_serialises_admission(server_cls, rng):
    # Each 2^18 u32 key-value sort needs ~4 MiB: a 6 MiB budget admits one at a time.
    n = 1 << 18
    srv = server_cls(budget_bytes=6 << 20, num_slots=4)
    reqs = []
    for _ in range(8):
        k = gen_keys(rng, n, np.uint32)
        v = np.arange(n, dtype=np.uint32)
        ok, ov = np.empty_like(k), np.empty_like(v)
        reqs.append((srv.submit_sort(k, v, ok, ov), k, ok, ov))
    srv.drain()
    st = srv.stats()
    assert st["completed"] == 8 and st["peak_bytes"] <= 6 << 20
    for rid, k, ok, ov in reqs:
        assert srv.poll(rid)
        order = np.argsort(k, kind="stable")
        assert np.array_equal(ok, k[order]) and np.array_equal(ov, order.astype(np.uint32))
    srv.close()


def test_empty_and_invalid_requests(server_cls, mgpu):
    srv = server_cls(budget_bytes=1 << 24, num_slots=2)
    e = np.empty(0, np.uint32)
    srv.wait(srv.submit_sort(e, None, e, None))
    srv.wait(srv.submit_merge(e, e, e, e, e, e))
    srv.wait(srv.submit_scan(e, e))
    with pytest.raises(mgpu.MgpuError):
        # Scan of a value-carrying request is not a request the server takes.
        req = mgpu.Request(op=2, key_type=1, val_bytes=4, count=4)
        srv.submit(req)
    with pytest.raises(mgpu.MgpuError):
        srv.wait(123456)            # never issued
    st = srv.stats()
    assert st["completed"] == 3 and st["failed"] == 0
    srv.close()


def test_latency_record(server_cls, rng):
    srv = server_cls(budget_bytes=1 << 28, num_slots=3)
    lats = []
    for _ in range(20):
        k = gen_keys(rng, 1 << 14, np.float32)
        ok = np.empty_like(k)
        lats.append(srv.wait(srv.submit_sort(k, None, ok, None)))
    st = srv.stats()
    assert st["completed"] == 20
    assert 0 < st["p50_ms"] <= st["p99_ms"] <= st["max_ms"]
    assert abs(st["max_ms"] - max(lats)) < 1e-6
    srv.reset_stats()
    assert srv.stats()["completed"] == 0
    srv.close()
