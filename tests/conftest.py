import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def orc():
    from oracle import pyoracle
    pyoracle.build()
    return pyoracle


@pytest.fixture(scope="session")
def smcgpu():
    """The CUDA library, built in-tree; GPU tests fail loudly if it is missing."""
    from smc_inversion_fort_gb300 import build
    build.build()
    import smc_inversion_fort_gb300 as pkg
    pkg.load_library()
    return pkg
