"""pytest configuration: the ``gpu`` marker and path setup.

Tests marked ``gpu`` need a CUDA device and call the library through its C ABI;
everything else runs on a CPU-only machine (oracle vs golden vectors, host
logic, ABI exports, multi-rank host logic on gloo).
"""

import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)
TESTS = os.path.dirname(os.path.abspath(__file__))
if TESTS not in sys.path:
    sys.path.insert(0, TESTS)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle

    oracle.lib()
    oracle.set_threads(1)
    return oracle
