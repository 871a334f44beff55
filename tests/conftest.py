import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")
STENCILS = ["star2d1r", "star2d2r", "box2d1r", "box2d2r"]


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def tcs():
    """The engine, built in-tree (no fallback: a missing build is an error)."""
    import tcstencil_gb300
    from tcstencil_gb300 import build

    build.build()
    tcstencil_gb300.lib()
    return tcstencil_gb300


@pytest.fixture(scope="session")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    return torch


@pytest.fixture(scope="session")
def golden():
    def load(name):
        return np.load(os.path.join(GOLDEN, name))
    return load
