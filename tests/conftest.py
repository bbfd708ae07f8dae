import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libpbf103.so")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def lib():
    """The CUDA library; built on demand (tests never fall back to a CPU path)."""
    from ssf_pbf_cuda_gb300 import build
    build.build()
    from ssf_pbf_cuda_gb300 import _lib
    return _lib.load()


@pytest.fixture(scope="session")
def gpu(lib):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected on a machine without a CUDA device")
    torch.cuda.init()
    return torch.device("cuda:0")
