"""Shared test configuration.

Tests marked ``gpu`` need a CUDA device and call the product through its C ABI;
everything else runs on the CPU (oracle pinning, host logic, ABI surface).
"""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running check")


@pytest.fixture(scope="session")
def oracle():
    from oracle import pyoracle
    pyoracle.build(ref=False)
    return pyoracle


@pytest.fixture(scope="session")
def golden():
    import numpy as np

    def load(name):
        return dict(np.load(GOLDEN / name, allow_pickle=False))

    return load


@pytest.fixture(scope="session")
def native():
    from devilray_gb300 import native as nat
    nat.load()
    return nat


@pytest.fixture(scope="session")
def ctx(native):
    return native.Context(0)
