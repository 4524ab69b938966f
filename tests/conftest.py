import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) and the built libdgpu.so")


def _has_sm103() -> bool:
    try:
        import torch
        return torch.cuda.is_available() and torch.cuda.get_device_capability(0) == (10, 3)
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu_lib():
    """Built and loaded libdgpu.so; GPU tests fail (not skip) when the device or library is missing."""
    import dpgsolver_gb300
    dpgsolver_gb300.build()
    lib = dpgsolver_gb300.load()
    if not _has_sm103():
        pytest.fail("GPU test needs an sm_103 device")
    return lib
