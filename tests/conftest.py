"""Shared test setup.

Marker ``gpu``: needs a CUDA device (GB300, sm_103).  CPU-only runs use
``-m "not gpu"``.
"""
from __future__ import annotations

import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: test needs a GB300 (sm_103) CUDA device")


def golden_names() -> list[str]:
    return sorted(os.path.splitext(os.path.basename(p))[0]
                  for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load_golden(name: str) -> dict:
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


@pytest.fixture(scope="session")
def gas_lib():
    """The in-tree C-ABI library, built on demand (nvcc cross-compiles)."""
    from vertexapi2_gb300 import build
    build.build()
    from vertexapi2_gb300 import _lib
    return _lib.load()


@pytest.fixture(scope="session")
def port():
    import oracle
    return oracle.port()


@pytest.fixture(scope="session")
def gpu(gas_lib):
    """Skips unless a supported GPU is present; the library must then load."""
    if not gas_lib.gas_device_supported(0):
        pytest.skip("no sm_103 device")
    return gas_lib
