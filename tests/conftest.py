import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")
    config.addinivalue_line("markers", "slow: long CPU-only oracle runs")


@pytest.fixture(scope="session")
def amx_lib():
    """The C-ABI library, built in-tree when it is missing or stale."""
    from astronomix_gb300 import _build, _native

    _build.build()
    return _native.lib()


@pytest.fixture(scope="session")
def cuda(amx_lib):
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test collected without a visible CUDA device")
    return torch.device("cuda")
