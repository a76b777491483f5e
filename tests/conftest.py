import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs an sm_103 (GB300) CUDA device")


@pytest.fixture(scope="session", autouse=True)
def _built_checker():
    """The CPU oracle is test infrastructure; build it once per session."""
    from oracle import lw
    lw.build(with_reference=True)
    yield


@pytest.fixture(scope="session")
def config1():
    from teufel_gb300 import harness
    return harness.config1()
