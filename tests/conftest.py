import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running")


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    d = os.path.join(ROOT, "tests", "golden")
    return {name: np.load(os.path.join(d, name + ".npz"))
            for name in ("integrate", "sweeps", "host", "models", "grad", "dfe", "settings",
                         "known")}


@pytest.fixture(scope="session")
def cuda_lib():
    """The built library on a visible CUDA device (gpu tests only)."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("gpu test collected without a CUDA device")
    from dadi_gb300 import _lib, build
    build.build()
    return _lib.lib()
