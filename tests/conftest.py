"""pytest configuration: the gpu marker and shared fixtures.

Tests marked gpu need a CUDA device and the built library; everything else
runs on the CPU (oracle against golden vectors, host-side logic, library
loading and exports).
"""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(Path(__file__).resolve().parent))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libmag2d_gpu.so")


@pytest.fixture(scope="session")
def built():
    """Build the CUDA library and the oracle port once per session."""
    import __graft_entry__

    __graft_entry__.build()
    return True
