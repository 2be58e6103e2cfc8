"""The C++ backend classes (include/vsmc_cuda_backend.hpp) compile and link
against the reference's own Sampler<T> headers.  Runs where the reference
tree is present; the binary itself needs a GPU to run."""
import os
import subprocess

import pytest

from conftest import ROOT

from oracle.binding import ref_root

REF = ref_root()


@pytest.mark.skipif(REF is None,
                    reason="reference headers not present on this host")
def test_backend_header_builds_against_reference_sampler(tmp_path):
    from vsmc_gb300 import build
    lib = build.build()
    cuda = "/usr/local/cuda"
    out = tmp_path / "backend_demo"
    cmd = ["g++", "-std=c++14", "-O1", "-w",
           "-I", os.path.join(REF, "include"),
           "-I", os.path.join(ROOT, "tests", "cpp", "shim"),
           "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(cuda, "include"),
           "-DVSMC_RNG_TYPE=::vsmc::Philox4x32", "-DVSMC_HAS_MKL=0",
           "-DVSMC_HAS_TBB=0",
           os.path.join(ROOT, "tests", "cpp", "backend_demo.cpp"),
           "-o", str(out), "-L", os.path.dirname(lib), "-lvsmc_cuda",
           "-L", os.path.join(cuda, "lib64"), "-lcudart",
           f"-Wl,-rpath,{os.path.dirname(lib)}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    assert out.exists()
