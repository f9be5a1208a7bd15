import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(Path(__file__).resolve().parent))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs an sm_103 GPU (GB300)")
    config.addinivalue_line("markers", "slow: long-running check")


@pytest.fixture(scope="session")
def cuda_ready():
    import torch
    from pycd_gb300 import _native as nat
    assert torch.cuda.is_available(), "GPU test run without a GPU"
    nat.require_device()
    return True
