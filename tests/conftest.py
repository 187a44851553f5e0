import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libflowmc.so")
    config.addinivalue_line("markers", "slow: long-running statistical test")


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from flowmc_gb300 import _lib
    _lib.lib()
    return torch.device("cuda")


@pytest.fixture(autouse=True)
def _seed_torch():
    """Every test starts from the same torch generator state (CPU and CUDA),
    so inputs drawn with torch.randn are the same on every run."""
    import torch
    torch.manual_seed(0)
