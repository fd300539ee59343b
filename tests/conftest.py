import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Both libraries are built in-tree before any test runs (cached by mtime)."""
    from oracle import oracle
    from trace_gb300 import build

    oracle.build()
    build.build()


@pytest.fixture(scope="session")
def ctx():
    from trace_gb300 import pt

    c = pt.Context(0)
    yield c
    c.close()
