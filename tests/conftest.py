import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def lib():
    from nemaktis_gb300 import _lib
    return _lib.load()


@pytest.fixture(scope="session")
def gpu(lib):
    if not has_gpu():
        pytest.skip("no CUDA device")
    return lib
