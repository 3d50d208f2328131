import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libcdx.so")


@pytest.fixture(scope="session")
def cdx():
    """The built C library through its ctypes binding (builds it when missing)."""
    from cdixx_gb300 import build, native
    if not native.LIB_PATH.exists():
        build.build()
    native.lib()
    return native


@pytest.fixture(scope="session")
def torch_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected without a CUDA device")
    return torch
