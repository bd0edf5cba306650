"""Shared pytest setup: the `gpu` marker, import paths, and helpers."""
import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


def interior(a: np.ndarray) -> np.ndarray:
    """Interior cells of a host-layout array (nz+4, ny+4, nx+4, neq)."""
    return a[2:-2, 2:-2, 2:-2]


@pytest.fixture(scope="session")
def gpu_lib():
    """The GB300 library, built in-tree if needed (fails loudly without it)."""
    from guacho_gb300 import build
    build.build()
    from guacho_gb300 import _abi
    return _abi.lib()
