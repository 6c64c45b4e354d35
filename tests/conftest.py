import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def built_lib():
    """Build (if stale) and return the path of liblbm_gb300.so."""
    from lb_gb300 import build
    return build.build()


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import build
    return build.build()
