"""Shared test set-up: the `gpu` marker, repo imports and the native build."""
import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = ROOT / "tests" / "golden"
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def native_build():
    """Builds libmantiis_gpu.so and the CPU oracle if they are not there yet."""
    from mantiis_gb300 import build as b
    from oracle import pyoracle

    if not b.LIB.exists():
        b.build()
    if not pyoracle.LIB.exists():
        pyoracle.build()


def load(name):
    return dict(np.load(GOLDEN / name))


@pytest.fixture(scope="session")
def fixture64():
    return load("fixture64.npz")
