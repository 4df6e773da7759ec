import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the qgx library")


@pytest.fixture(scope="session")
def qgx_built():
    """Build libqgx.so in-tree when it is missing or stale (nvcc is on the GPU machine too)."""
    from quantax_gb300 import _build
    _build.build()
    return _build.LIB


@pytest.fixture(scope="session")
def cuda(qgx_built):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    torch.cuda.init()
    return torch.device("cuda", 0)
