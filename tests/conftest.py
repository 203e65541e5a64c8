"""Test configuration. Tests marked `gpu` need a CUDA device and call the library
through its C ABI; everything else runs on the CPU (the oracle against the
golden vectors, host-side logic, and the library's exported symbols)."""

from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(Path(__file__).resolve().parent))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU; calls the library through its C ABI")


@pytest.fixture(scope="session")
def device():
    from diorama_gb300 import Device

    dev = Device(0)
    yield dev
    dev.check()
    dev.destroy()


@pytest.fixture(scope="session")
def golden():
    return ROOT / "tests" / "golden"
