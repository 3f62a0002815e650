import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import __graft_entry__ as entry  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    O = entry.load_oracle()
    O.build()
    return O


@pytest.fixture(scope="session")
def pkg():
    """The package with libgfgb300.so built in-tree (nvcc cross-compiles on CPU)."""
    return entry.build()


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
