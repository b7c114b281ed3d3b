import os
import sys
import zlib

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (REPO, os.path.join(REPO, "mgpu-shaders_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: full-size workload")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as o
    o.lib()
    return o


@pytest.fixture(scope="session")
def mgpu():
    import mgpu_gb300
    mgpu_gb300.lib()
    return mgpu_gb300


@pytest.fixture(scope="session")
def ctx(mgpu):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    c = mgpu.Context(0)
    yield c
    c.synchronize()
    c.close()


@pytest.fixture
def rng(request):
    """A generator seeded by the test's id (crc32, so every run of a test
    draws the same inputs, unlike the per-process salted str hash)."""
    seed = zlib.crc32(request.node.nodeid.encode())
    return np.random.default_rng(seed)
