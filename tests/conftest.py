import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs through the C ABI on the device)")


@pytest.fixture(scope="session")
def torch_cuda():
    """torch with a CUDA device; GPU tests fail loudly if it is missing."""
    import torch
    assert torch.cuda.is_available(), "GPU test run without a CUDA device"
    return torch


@pytest.fixture(scope="session")
def gb300():
    """The CUDA library, built in-tree; no fallback."""
    import isar_imaging_cuda_gb300 as g
    g.load()
    return g
