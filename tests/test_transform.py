"""C ABI element-wise transforms (vk::transform's example operations,
examples/vk_transform/vk_transform.cxx:36-63) against numpy."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dt", [np.int32, np.uint32, np.float32, np.int64, np.uint64, np.float64])
@pytest.mark.parametrize("n", [0, 1, 1000, 3_000_001])
def test_iota_fill(mgpu, ctx, dt, n):
    d = mgpu.DeviceArray(n, dt)
    ctx.transform_iota(d, 3, 2)
    ctx.synchronize()
    assert np.array_equal(d.numpy(), (3 + 2 * np.arange(n)).astype(dt))
    ctx.transform_fill(d, 9)
    ctx.synchronize()
    assert np.array_equal(d.numpy(), np.full(n, 9, dt))


def test_saxpy(mgpu, ctx, rng):
    n = 1_000_003
    x = rng.standard_normal(n).astype(np.float32)
    y = rng.standard_normal(n).astype(np.float32)
    dx, dy = mgpu.DeviceArray.from_numpy(x), mgpu.DeviceArray.from_numpy(y)
    ctx.transform_saxpy(1.618, dx, dy)
    ctx.synchronize()
    ref = y + np.float32(1.618) * x
    assert np.allclose(dy.numpy(), ref, rtol=1e-6, atol=1e-6)
