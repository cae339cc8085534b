"""Shared fixtures.  ``-m gpu`` tests need a CUDA device and the built engine;
everything else runs on the CPU (oracle, host logic, C-ABI exports)."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GB300 device and the built engine")


@pytest.fixture(scope="session")
def engine():
    """The engine library (built in-tree on first use)."""
    import ttv_gb300
    if not os.path.exists(ttv_gb300.library_path()):
        from ttv_gb300 import build
        build.build()
    return ttv_gb300


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def cuda(engine):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    return torch.device("cuda:0")
