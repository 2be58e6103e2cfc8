"""The C-ABI library builds for sm_103a, loads, and exports every entry point
include/vsmc_cuda.h declares (no GPU work)."""
import ctypes
import os
import re
import subprocess

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "vsmc_cuda.h")


def declared():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(vsmc_cuda_\w+)\s*\(", src)))


@pytest.fixture(scope="module")
def libpath():
    from vsmc_gb300 import build
    return build.build()


def test_library_exports_every_declared_symbol(libpath):
    names = declared()
    assert len(names) > 40
    out = subprocess.run(["nm", "-D", "--defined-only", libpath],
                         capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT\s+(vsmc_cuda_\w+)", out))
    missing = [n for n in names if n not in exported]
    assert not missing, missing


def test_library_loads_and_binding_covers_header(libpath):
    import vsmc_gb300
    L = ctypes.CDLL(libpath)
    for n in declared():
        assert hasattr(L, n), n
        assert n in vsmc_gb300.PROTOTYPES, f"no ctypes prototype for {n}"


def test_build_targets_sm103a_only():
    from vsmc_gb300 import build
    flags = " ".join(build.NVCC_FLAGS)
    assert "arch=compute_103a,code=sm_103a" in flags
    assert flags.count("-gencode") == 1


def test_host_side_status_and_engine_setup(libpath):
    """Pure host entry points: status strings and engine placement."""
    import vsmc_gb300 as vc
    assert vc.lib().vsmc_cuda_status_string(vc.ERR_ARG) == b"invalid argument"
    assert vc.lib().vsmc_cuda_version() >= 100
    r = vc.rng(vc.PHILOX4X32, seed=0xFFFFFFFFFFFF)
    assert r.key[0] == 0xFFFFFFFF and r.index == 4   # 32-bit key limbs
    r = vc.rng(vc.THREEFRY4X64, key=[1, 2, 3, 4], ctr=[5, 6])
    assert list(r.key) == [1, 2, 3, 4] and list(r.ctr) == [5, 6, 0, 0]
    assert r.index == 4
    # bad arguments are rejected before any device work
    assert vc.lib().vsmc_cuda_rng_init(None, 0, 0) == vc.ERR_ARG
    h = ctypes.c_void_p()
    m = vc.default_model()
    assert vc.lib().vsmc_cuda_pf_create(ctypes.byref(h), 0, 32, 2, 0.5, 0,
                                        ctypes.byref(m), 10, None) == vc.ERR_SIZE
    assert vc.lib().vsmc_cuda_pf_create(ctypes.byref(h), 10, 16, 2, 0.5, 0,
                                        ctypes.byref(m), 10, None) == vc.ERR_ARG
    bad = vc.CvModel(0.1, 1.0, -0.5, 10.0, 2.0, 1.0)
    assert vc.lib().vsmc_cuda_pf_create(ctypes.byref(h), 10, 32, 2, 0.5, 0,
                                        ctypes.byref(bad), 10, None) == vc.ERR_ARG


def test_batch_create_validates_before_device_work():
    import ctypes
    import numpy as np
    import vsmc_gb300 as vc
    L = vc.lib()
    h = ctypes.c_void_p()
    m = (vc.CvModel * 2)(vc.default_model(), vc.default_model())
    T = np.array([5, 5], np.uint32)
    seeds = np.array([1, 2], np.uint32)
    bad_n = np.array([1, 10], np.uint32)
    assert L.vsmc_cuda_batch_create(ctypes.byref(h), 2, bad_n.ctypes.data,
                                    T.ctypes.data, m, seeds.ctypes.data, 1,
                                    0.5, None) == vc.ERR_SIZE
    n = np.array([10, 10], np.uint32)
    assert L.vsmc_cuda_batch_create(ctypes.byref(h), 2, n.ctypes.data,
                                    T.ctypes.data, m, seeds.ctypes.data, 0,
                                    0.5, None) == vc.ERR_ARG
    assert L.vsmc_cuda_batch_create(ctypes.byref(h), 0, n.ctypes.data,
                                    T.ctypes.data, m, seeds.ctypes.data, 1,
                                    0.5, None) == vc.ERR_SIZE
