"""Test configuration: the ``gpu`` marker and import paths.

Tests marked ``gpu`` need a CUDA device and call the product through its C
ABI; everything else runs on the CPU (oracle checks, host logic, the
library's exported symbols).
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "opm-models_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session")
def built():
    """Build the CUDA library and the oracle once per session."""
    import __graft_entry__ as ge
    ge.build()
    return True
