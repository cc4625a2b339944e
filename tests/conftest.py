"""Shared test setup: the `gpu` marker and import paths.

Tests marked ``gpu`` need a CUDA device and call the native library through its
C ABI; everything else runs on the CPU (oracle against golden fixtures, host
logic, library loading and exported symbols).
"""

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    import numpy as np

    def load(name):
        return np.load(GOLDEN / name)

    return load
