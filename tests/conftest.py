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


_KEEP = []


def dev(a):
    """numpy -> CUDA tensor (same dtype).

    The tensor is also kept in a per-test list: `dev(x).data_ptr()` passed
    straight to a C call would otherwise let the temporary be freed at once,
    and the caching allocator could hand the same block to the next dev()."""
    import torch
    t = torch.from_numpy(np.ascontiguousarray(a)).cuda()
    _KEEP.append(t)
    return t


@pytest.fixture(autouse=True)
def _release_kept_tensors():
    yield
    _KEEP.clear()


def host(t):
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy()
