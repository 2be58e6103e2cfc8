"""Shared fixtures.  GPU tests are marked `gpu`; everything else runs on CPU."""
import ctypes
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def port():
    from oracle import binding
    return binding.port()


@pytest.fixture(scope="session")
def vc():
    """The vsmc_gb300 module with libvsmc_cuda loaded (GPU tests only)."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected without a CUDA device")
    import vsmc_gb300
    vsmc_gb300.lib()
    return vsmc_gb300


def P(a):
    """ctypes pointer of a numpy array."""
    return a.ctypes.data_as(ctypes.c_void_p)


def dev(a):
    """numpy -> CUDA tensor (same dtype)."""
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy()
