import os
import sys

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
    seed = abs(hash(request.node.nodeid)) % (2 ** 32)
    return np.random.default_rng(seed)
