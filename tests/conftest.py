"""Shared pytest configuration.

Tests marked `gpu` need a CUDA device (they call libgrus through its C ABI);
everything else runs on the CPU: the oracle against the golden fixtures, the
host logic, and the C-ABI library's exports (no compute calls).
"""
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libgrus.so")
    config.addinivalue_line("markers", "slow: larger configurations (seconds of oracle time)")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build.build_oracle()
    return oracle


@pytest.fixture(scope="session")
def grus():
    """The product package, built if needed, with device 0 initialised."""
    from grus_framework_gb300 import build as b
    b.build()
    import grus_framework_gb300 as g
    g.device_init(0)
    return g
