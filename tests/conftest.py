"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on
the CPU (the oracle, host-side logic, and that the C-ABI library loads)."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libgwlnl.so")
    config.addinivalue_line("markers", "reference: needs the reference source tree (skipped where absent)")


def cuda_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu():
    """Skip nothing silently on a GPU machine: if the mark says gpu, CUDA must be there."""
    if not cuda_available():
        pytest.skip("no CUDA device")
    from bilby_gb300 import _build
    _build.build()
    return True


def golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))
