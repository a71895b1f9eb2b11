"""Shared fixtures.  GPU tests carry @pytest.mark.gpu and call the CUDA
library through its C ABI; the CPU suite checks the oracle, the host-side
code and the library's exports."""
import importlib
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def cpmp():
    """The package, with libcpmp.so built in-tree."""
    build = importlib.import_module("3dcpmpmodel_gb300.build")
    build.build()
    return importlib.import_module("3dcpmpmodel_gb300")
