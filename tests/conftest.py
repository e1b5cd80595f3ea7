import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the librgdn kernels")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds the native libraries once per session (incremental, seconds)."""
    from raytracedgl1_gb300 import build
    build.build_all()
    yield


@pytest.fixture(scope="session")
def cuda_ok():
    try:
        import torch
        ok = torch.cuda.is_available()
    except Exception:
        ok = False
    if not ok:
        pytest.skip("no CUDA device")
    return True


@pytest.fixture(scope="session")
def ctx(cuda_ok):
    from raytracedgl1_gb300.denoiser import Context
    c = Context(0)
    yield c
    c.close()
