import glob
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)



def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


def _has_gpu_device():
    return os.path.exists("/dev/nvidiactl") or bool(glob.glob("/dev/nvidia[0-9]*"))


def pytest_collection_modifyitems(config, items):
    if _has_gpu_device():
        return
    skip = pytest.mark.skip(reason="no NVIDIA device on this machine")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session", autouse=True)
def native_built():
    """Builds the library and the oracle once per session (incremental)."""
    from spinwalk_gb300 import _build
    _build.build_all()


