import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libappfis_gb.so")
    config.addinivalue_line("markers", "slow: large CPU case")


@pytest.fixture(scope="session")
def gb():
    """The C-ABI library, built if needed; GPU tests only."""
    from appfis_gb300 import build
    build.build()
    import appfis_gb300
    return appfis_gb300


@pytest.fixture(scope="session")
def torch_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("a GPU test ran without a visible CUDA device")
    torch.cuda.init()
    return torch
