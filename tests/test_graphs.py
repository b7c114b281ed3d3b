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
