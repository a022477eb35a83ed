import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA library")
    config.addinivalue_line("markers", "slow: full-size case (seconds to a minute)")


@pytest.fixture(scope="session")
def cuda_lib():
    """The built CUDA library; GPU tests fail (not skip) when it is missing."""
    from maestro_gb300 import capi
    from maestro_gb300.build import build
    build()
    return capi.lib()
