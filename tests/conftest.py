import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a)")


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu():
    if not has_gpu():
        pytest.skip("no CUDA device")
    import torch
    from ironclust_gb300 import build
    build.build()
    return torch.device("cuda:0")


@pytest.fixture(scope="session")
def refk(gpu):
    """The reference's own kernels (PTX compiled from its sources)."""
    from oracle.oracle import RefKernels
    return RefKernels()
