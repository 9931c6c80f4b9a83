"""Shared test setup.

Marker `gpu`: needs a CUDA device (run with -m gpu on a GB300); everything else
runs on the CPU.  The CPU oracle (oracle/) is the checker in every parity test.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")
if GOLDEN not in sys.path:
    sys.path.insert(0, GOLDEN)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: requires a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import build, lib

    build.build()
    return lib


@pytest.fixture(scope="session")
def gcq():
    """The libgcq.so binding; builds the library if needed.  GPU tests only."""
    import gcq_gb300
    from gcq_gb300 import build

    if not os.path.exists(gcq_gb300.LIB_PATH):
        build.build()
    gcq_gb300.lib()
    return gcq_gb300
