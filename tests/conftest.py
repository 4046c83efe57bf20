"""Shared fixtures.  `-m gpu` tests need a GB300 and call libgba through its
C ABI; everything else runs on the CPU (oracle, host code, library load)."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running case")


@pytest.fixture(scope="session", autouse=True)
def built():
    """Builds libgba.so and the CPU oracle once per session (incremental)."""
    from slamplay_gb300 import build as B
    B.build()
    from oracle import oracle_py
    oracle_py.ensure_built(reference=False)
    return True
