import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: takes more than a few seconds")


@pytest.fixture(scope="session")
def gpu_libs():
    """Builds (if needed) and loads the native libraries; the GPU tests call
    through their C-ABI.  Fails -- never skips -- when the engine cannot load."""
    import xfdtd_gb300
    xfdtd_gb300.build()
    return xfdtd_gb300.libs()
