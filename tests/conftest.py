"""Shared test configuration.

Tests marked ``gpu`` need a CUDA device and the built library; everything
else runs on the CPU (oracle vs golden vectors, host logic, ABI symbols).
"""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built phrike_gb300 library")


@pytest.fixture(scope="session")
def built_lib():
    """Build (if stale) and load the CUDA library."""
    from phrike_gb300 import _build, _lib
    _build.build()
    return _lib.load()


@pytest.fixture(scope="session")
def cuda_device(built_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    return torch.device("cuda", 0)


def golden(name):
    import numpy as np
    return np.load(os.path.join(GOLDEN, name))


def rel_l2(a, b):
    import numpy as np
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))
