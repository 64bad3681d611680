"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on the
CPU.  The oracle (oracle/port) is the checker only."""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the libgbode kernels)")


@pytest.fixture(scope="session")
def port():
    from oracle.port.port import Port
    return Port()


@pytest.fixture(scope="session")
def golden():
    def load(name):
        return np.load(os.path.join(GOLDEN, name))
    return load


@pytest.fixture(scope="session")
def gblib():
    """libgbode, built for sm_103a and loaded; GPU tests only."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    from ode_gb300 import build, ode
    build.build()
    return ode.load()
