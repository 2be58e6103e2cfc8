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


_M32 = np.uint64(0xFFFFFFFF)


def philox4x32_10(c, k0, k1):
    """Vectorized Philox4x32-10 block function (the Random123 generator of
    rng/philox.hpp:162-294, no pre-increment) on 32-bit words held in
    uint64 arrays; c is four counter words (arrays of equal length)."""
    c0, c1, c2, c3 = (np.asarray(v, np.uint64) & _M32 for v in c)
    k0 = np.uint64(k0)
    k1 = np.uint64(k1)
    for r in range(10):
        if r > 0:
            k0 = (k0 + np.uint64(0x9E3779B9)) & _M32
            k1 = (k1 + np.uint64(0xBB67AE85)) & _M32
        pa = c2 * np.uint64(0xCD9E8D57)
        pb = c0 * np.uint64(0xD2511F53)
        n0 = (pa >> np.uint64(32)) ^ k0 ^ c1
        n2 = (pb >> np.uint64(32)) ^ k1 ^ c3
        c0, c1, c2, c3 = n0 & _M32, pa & _M32, n2 & _M32, pb & _M32
    return c0, c1, c2, c3


def particle_words(t, seed, n, block=1):
    """The four words of block `block` of every particle's stream at step
    t: Philox4x32 key {t, seed}, counter {block, i, 0, 0}."""
    i = np.arange(n, dtype=np.uint64)
    z = np.zeros(n, np.uint64)
    return philox4x32_10([np.full(n, block, np.uint64), i, z, z], t, seed)


def normal_pair_f64(w0, w1):
    """Box-Muller in float64 on the FP32 kernels' own uniforms: a 24-bit
    (0, 1] radius uniform and a 24-bit [0, 1) angle uniform."""
    u1 = ((w0 >> np.uint64(8)).astype(np.float64) + 1) * 2.0**-24
    u2 = (w1 >> np.uint64(8)).astype(np.float64) * 2.0**-24
    r = np.sqrt(-2 * np.log(u1))
    return r * np.cos(2 * np.pi * u2), r * np.sin(2 * np.pi * u2)
