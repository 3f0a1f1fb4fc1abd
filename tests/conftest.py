"""Shared fixtures: the GPU marker, library builds and the oracle."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session", autouse=True)
def _built_libraries():
    """Compile the oracle (g++, seconds) and, if missing, the CUDA library."""
    from oracle import oracle as orc
    orc.build()
    from saras_gb300 import _abi
    if not os.path.exists(_abi.LIB_PATH):
        from saras_gb300.build import build
        build()
    yield


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
