"""CUDA-graph capture of multi-launch pipelines through the C ABI: a radix
sort (memset + histogram + 4 passes) and a mergesort captured once and
replayed on new data must give the oracle's results."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture
def gctx(mgpu):
    """A context on its own (capturable, non-default) stream."""
    c = mgpu.Context(0, use_torch_stream=False)
    yield c
    c.synchronize()
    c.close()


def test_radix_sort_graph_replay(mgpu, gctx, oracle, rng):
    ctx = gctx
    import torch
    n = 1_000_003
    dk = mgpu.DeviceArray(n, np.uint32)
    dv = mgpu.DeviceArray(n, np.uint32)
    size = ctx.radix_sort_aux_size(np.uint32, np.uint32, n)
    aux = torch.empty(size, dtype=torch.uint8, device="cuda")
    ctx.synchronize()
    ctx.graph_begin()
    ctx.radix_sort(dk, dv, aux=(aux.data_ptr(), size))
    g = ctx.graph_end()
    for _ in range(3):
        k = rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
        v = np.arange(n, dtype=np.uint32)
        dk.copy_from(mgpu.DeviceArray.from_numpy(k))
        dv.copy_from(mgpu.DeviceArray.from_numpy(v))
        torch.cuda.synchronize()
        g.launch()
        ctx.synchronize()
        ok, ov = oracle.radix_sort(k, v)
        assert np.array_equal(dk.numpy(), ok) and np.array_equal(dv.numpy(), ov)
    g.close()


def test_radix_sort_graph_count_on_device(mgpu, gctx, oracle, rng):
    """One graph captured at a capacity replays for any count written to
    device memory between replays; elements past the count stay as they
    are."""
    ctx = gctx
    import torch
    cap = 400_000
    dk = mgpu.DeviceArray(cap, np.uint32)
    dv = mgpu.DeviceArray(cap, np.uint32)
    dcount = torch.zeros(1, dtype=torch.int64, device="cuda")
    size = ctx.radix_sort_aux_size(np.uint32, np.uint32, cap)
    aux = torch.empty(size, dtype=torch.uint8, device="cuda")
    ctx.synchronize()
    ctx.graph_begin()
    ctx.radix_sort(dk, dv, aux=(aux.data_ptr(), size), device_count=dcount.data_ptr())
    g = ctx.graph_end()
    for count in (cap, 1, 0, 5120, 5121, 77_777, cap - 3):
        k = rng.integers(0, 2 ** 32, cap, dtype=np.uint64).astype(np.uint32)
        v = np.arange(cap, dtype=np.uint32)
        dk.copy_from(mgpu.DeviceArray.from_numpy(k))
        dv.copy_from(mgpu.DeviceArray.from_numpy(v))
        dcount.fill_(count)
        torch.cuda.synchronize()
        g.launch()
        ctx.synchronize()
        ok, ov = oracle.radix_sort(k[:count], v[:count])
        gk, gv = dk.numpy(), dv.numpy()
        assert np.array_equal(gk[:count], ok) and np.array_equal(gv[:count], ov), count
        assert np.array_equal(gk[count:], k[count:]) and np.array_equal(gv[count:], v[count:])
    # A count above the capacity is clamped to it.
    k = rng.integers(0, 2 ** 32, cap, dtype=np.uint64).astype(np.uint32)
    dk.copy_from(mgpu.DeviceArray.from_numpy(k))
    dcount.fill_(cap + 12345)
    torch.cuda.synchronize()
    g.launch()
    ctx.synchronize()
    assert np.array_equal(dk.numpy(), np.sort(k))
    g.close()


def test_mergesort_graph_with_reserved_cache(mgpu, gctx, oracle, rng):
    ctx = gctx
    import torch
    n = 300_001
    dk = mgpu.DeviceArray(n, np.int32)
    dv = mgpu.DeviceArray(n, np.uint32)
    ctx.cache_reserve(64 << 20)
    ctx.synchronize()
    ctx.graph_begin()
    ctx.mergesort(dk, dv)            # aux from the (already large enough) cache
    g = ctx.graph_end()
    for _ in range(2):
        k = rng.integers(0, 1000, n).astype(np.int32)
        v = np.arange(n, dtype=np.uint32)
        dk.copy_from(mgpu.DeviceArray.from_numpy(k))
        dv.copy_from(mgpu.DeviceArray.from_numpy(v))
        torch.cuda.synchronize()
        g.launch()
        ctx.synchronize()
        ok, ov = oracle.sort(k, v)
        assert np.array_equal(dk.numpy(), ok) and np.array_equal(dv.numpy(), ov)
    g.close()


def test_capture_rejects_cache_growth(mgpu, gctx):
    ctx = gctx
    n = 1 << 26
    dk = mgpu.DeviceArray(n, np.uint32)
    ctx.synchronize()
    ctx.graph_begin()
    with pytest.raises(mgpu.MgpuError):
        ctx.radix_sort(dk)            # would need to grow the cache inside the capture
    g = ctx.graph_end()
    g.close()
