import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs through libnmmc's C ABI)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds libnmmc and the oracle once per session (no-ops when up to date)."""
    from nanomagmc_gb300 import build as libbuild
    from oracle import build as orbuild

    libbuild.build()
    orbuild.build()
    yield
