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


def bench_mix_requests(rng, n_req, max_log2):
    """The serving benchmark's mix, bounded for test time: sort / merge / scan
    in turn, sizes log-uniform in [2^10, 2^max_log2], keys u32 / u64 / f32 at
    50/25/25 %, sorts and merges carrying u32 values, integer scans exclusive
    and f32 scans inclusive."""
    reqs = []
    for i in range(n_req):
        n = int(2 ** rng.uniform(10, max_log2))
        kt = [np.uint32, np.uint32, np.uint64, np.float32][rng.integers(0, 4)]
        kind = ("sort", "merge", "scan")[i % 3]
        if kind == "sort":
            reqs.append(("sort", gen_keys(rng, n, kt), np.arange(n, dtype=np.uint32)))
        elif kind == "merge":
            na = n // 2
            a, b = np.sort(gen_keys(rng, na, kt)), np.sort(gen_keys(rng, n - na, kt))
            reqs.append(("merge", a, np.arange(na, dtype=np.uint32), b,
                         np.arange(n - na, dtype=np.uint32) + na))
        else:
            x = rng.standard_normal(n).astype(np.float32) if kt == np.float32 else \
                rng.integers(0, 1 << 20, n).astype(kt)
            reqs.append(("scan", x, "inc" if kt == np.float32 else "exc"))
    return reqs


def run_alone(server_cls, reqs):
    srv = server_cls(budget_bytes=1 << 31, num_slots=1)
    outs = []
    for r in reqs:
        rid, o = submit(srv, r)
        srv.wait(rid)
        outs.append(o)
    assert srv.stats()["coalesced"] == 0
    srv.close()
    return outs


def test_bench_mix_equals_alone(server_cls, oracle, rng):
    # The benchmark's key types and operations at sizes up to 2^22, all queued
    # at once: every result is byte-identical to the request served alone, and
    # to the oracle.  f32 scans are checked against the float64 oracle within
    # the bound of the scan tests: the scan's look-back adds tile aggregates
    # in an order that depends on timing, so their last bits vary by run.
    reqs = bench_mix_requests(rng, 60, 22)
    alone = run_alone(server_cls, reqs)
    srv = server_cls(budget_bytes=1 << 30, num_slots=4)
    pending = [submit(srv, r) for r in reqs]
    for rid, _ in pending:
        srv.wait(rid)
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    for r, a, (_, m) in zip(reqs, alone, pending):
        if r[0] == "scan" and r[1].dtype == np.float32:
            ref = np.cumsum(r[1].astype(np.float64))
            tol = 1e-4 * np.abs(r[1]).astype(np.float64).sum() + 1e-6
            assert np.max(np.abs(m[0] - ref)) <= tol
            assert np.max(np.abs(a[0] - ref)) <= tol
        else:
            assert same(a[0], m[0]) and same(a[1], m[1]), (r[0], r[1].dtype, r[1].size)
            ek, ev = expected(oracle, r)
            assert same(ek, m[0]) and same(ev, m[1]), r[0]


def small_requests(rng, n_req):
    """Small sorts (keys only and key-value), merges (u32 keys, which coalesce
    with the u32 sorts, and f32 keys, which run alone) and integer scans of a
    few kinds, interleaved, sizes 1 .. 2^16 (the coalescing limit)."""
    reqs = []
    for i in range(n_req):
        n = int(2 ** rng.uniform(0, 16))
        if i % 7 == 6:
            n = 1 << 16
        c = i % 6
        if c == 0:
            reqs.append(("sort", gen_keys(rng, n, np.uint32), np.arange(n, dtype=np.uint32)))
        elif c == 1:
            reqs.append(("sort", gen_keys(rng, n, np.float32), None))
        elif c == 2:
            reqs.append(("scan", rng.integers(0, 1 << 20, n).astype(np.int32), "exc"))
        elif c == 3:
            reqs.append(("scan", rng.integers(0, 1 << 40, n).astype(np.uint64), "inc"))
        else:
            kt = np.uint32 if c == 4 else np.float32
            na = n // 2
            # Few distinct keys, so A and B share many and the A-first rule shows.
            a = np.sort(gen_keys(rng, na, kt, "distinct256"))
            b = np.sort(gen_keys(rng, n - na, kt, "distinct256"))
            reqs.append(("merge", a, np.arange(na, dtype=np.uint32), b,
                         np.arange(n - na, dtype=np.uint32) + (1 << 30)))
    return reqs


def test_small_requests_coalesce(server_cls, oracle, rng):
    # 200 small requests queued behind one large sort that holds the only
    # slot: the queue fills, and the small ones run in coalesced batches (one
    # segmented sort or scan per batch; u32 merges as sort segments) with the
    # same bytes as alone.
    reqs = small_requests(rng, 200)
    alone = run_alone(server_cls, reqs)
    srv = server_cls(budget_bytes=1 << 30, num_slots=1)
    big = gen_keys(rng, 1 << 22, np.uint32)
    big_out = np.empty_like(big)
    first = srv.submit_sort(big, None, big_out, None)
    pending = [submit(srv, r) for r in reqs]
    srv.wait(first)
    for rid, _ in pending:
        srv.wait(rid)
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(reqs) + 1 and st["failed"] == 0
    assert st["coalesced"] >= len(reqs) // 2 and 0 < st["batches"] < st["coalesced"]
    assert np.array_equal(big_out, np.sort(big))
    for r, a, (_, m) in zip(reqs, alone, pending):
        assert same(a[0], m[0]) and same(a[1], m[1]), (r[0], r[1].dtype, r[1].size)
        ek, ev = expected(oracle, r)
        assert same(ek, m[0]) and same(ev, m[1]), r[0]


def test_coalescing_respects_budget(server_cls, oracle, rng):
    # A budget that holds only part of a batch: batches shrink to fit or the
    # requests run alone; nothing exceeds the budget and every result is right.
    reqs = small_requests(rng, 64)
    srv = server_cls(budget_bytes=2 << 20, num_slots=2)
    pending = [submit(srv, r) for r in reqs]
    for rid, _ in pending:
        srv.wait(rid)
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert st["peak_bytes"] <= 2 << 20
    for r, (_, m) in zip(reqs, pending):
        ek, ev = expected(oracle, r)
        assert same(ek, m[0]) and same(ev, m[1]), r[0]
