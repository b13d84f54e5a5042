import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and libmpc_gpu.so")
    config.addinivalue_line("markers", "slow: long-running CPU case")


@pytest.fixture(scope="session")
def gpu_lib():
    """Build (if needed) and load libmpc_gpu.so; the GPU tests call through its C ABI."""
    from mpc_gb300 import build, capi
    build.build()
    return capi.load()
