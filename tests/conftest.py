"""Shared test setup: the repository root on sys.path and the ``gpu`` marker."""

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libmeepgb.so")


def cuda_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:  # pragma: no cover
        return False


@pytest.fixture(scope="session")
def gpu():
    if not cuda_available():
        pytest.fail("this test is marked gpu and needs a CUDA device")
    import torch
    return torch.device("cuda", 0)
