import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GB300 device")
    config.addinivalue_line("markers", "slow: long-running parity case")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds the oracle and the CPU helper library once per session (the shipped library is
    built by __graft_entry__.build(); GPU tests need it)."""
    from oracle import build as ob
    ob.build()
    import __graft_entry__ as ge
    ge._build_test_helpers()
