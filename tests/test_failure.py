"""The failure path of the bounded device-side waits, exercised without a GPU
fault: a self-test kernel waits on an mbarrier phase and on a flag that
nothing completes, and the production radix pass runs a look-back on a
predecessor that never publishes; the waits give up after a short limit, the
context reports MGPU_ERR_LOOKBACK_TIMEOUT at the next synchronize, and the
context keeps working afterwards."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bounded_wait_reports_timeout_and_context_recovers(mgpu, oracle, rng):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ctx = mgpu.Context(0, use_torch_stream=False)
    ctx.selftest_bounded_wait(2048)
    with pytest.raises(mgpu.MgpuError) as e:
        ctx.synchronize()
    assert e.value.status == 3
    ctx.synchronize()                     # the error word was cleared
    # The context still sorts correctly.
    n = 100_003
    k = rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
    v = np.arange(n, dtype=np.uint32)
    dk, dv = mgpu.DeviceArray.from_numpy(k), mgpu.DeviceArray.from_numpy(v)
    torch.cuda.synchronize()
    ctx.radix_sort(dk, dv)
    ctx.synchronize()
    ok, ov = oracle.radix_sort(k, v)
    assert np.array_equal(dk.numpy(), ok) and np.array_equal(dv.numpy(), ov)
    ctx.close()


def test_bounded_wait_limit_is_checked(mgpu):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ctx = mgpu.Context(0, use_torch_stream=False)
    for bad in (0, -1, (1 << 22) + 1):
        with pytest.raises(mgpu.MgpuError) as e:
            ctx.selftest_bounded_wait(bad)
        assert e.value.status == 1
    ctx.close()


def test_radix_lookback_timeout_reports_and_context_recovers(mgpu, oracle, rng):
    # The production onesweep pass, its tile counter advanced past tile 0: the
    # real decoupled look-back waits on a row nobody publishes, gives up after
    # the context's short wait limit, and the context reports status 3 once.
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ctx = mgpu.Context(0, use_torch_stream=False)
    ctx.set_wait_limit(4096)
    ctx.selftest_lookback_timeout()
    with pytest.raises(mgpu.MgpuError) as e:
        ctx.synchronize()
    assert e.value.status == 3
    ctx.synchronize()                     # the error word was cleared
    # With the library's limit restored the same context sorts exactly.
    ctx.set_wait_limit(0)
    n = 1_000_003
    k = rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
    v = np.arange(n, dtype=np.uint32)
    dk, dv = mgpu.DeviceArray.from_numpy(k), mgpu.DeviceArray.from_numpy(v)
    torch.cuda.synchronize()
    ctx.radix_sort(dk, dv)
    ctx.synchronize()
    ok, ov = oracle.radix_sort(k, v)
    assert np.array_equal(dk.numpy(), ok) and np.array_equal(dv.numpy(), ov)
    ctx.close()


def test_wait_limit_is_checked(mgpu):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ctx = mgpu.Context(0, use_torch_stream=False)
    for bad in (-1, (1 << 22) + 1):
        with pytest.raises(mgpu.MgpuError) as e:
            ctx.set_wait_limit(bad)
        assert e.value.status == 1
    ctx.close()
