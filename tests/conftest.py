import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    return dict(np.load(os.path.join(ROOT, "tests", "golden", "env_rob.npz")))


@pytest.fixture(scope="session")
def gpu_lib():
    """Initialises the native library on cuda:0 (GPU tests only)."""
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from fcl_gb300 import native
    L = native.lib()
    native.check(L.fclgpu_init(0), "fclgpu_init")
    return L
