import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)


def pytest_configure(config):
    config.addinivalue_line(
        "markers", "gpu: needs a CUDA GPU (GB300) and the built libphase_gb300")


@pytest.fixture(scope="session")
def oracle():
    import oracle_bind
    oracle_bind.lib()
    return oracle_bind


@pytest.fixture(scope="session")
def pg():
    """The product library (GPU tests only)."""
    import __graft_entry__
    __graft_entry__.build()
    import phase_gb300
    phase_gb300.lib()
    return phase_gb300
