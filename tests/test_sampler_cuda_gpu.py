"""vSMC's own Sampler<T> driving the fused FP32 CUDA backend.

tests/cpp/sampler_cuda.cu is compiled with nvcc against the reference's
headers (found through oracle.binding.ref_root(): VSMC_REF_ROOT or the
reference checkout; the test is skipped where neither exists) and runs
Sampler<StateCUDA<4, float>> with InitializeCUDA / MoveCUDA of a user device
model, MonitorMeanCUDA and WeightCUDAF32 (include/vsmc_cuda_sampler.cuh):
Sampler::initialize / iterate (core/sampler.hpp:443-476, 735-785) calling
Particle::resample (core/particle.hpp:170-197) and Monitor::eval
(core/monitor.hpp:242-268) exactly as with the reference's CPU backends.

Its histories (the Sampler's ESS and resampled records, the monitor's
records, the weight's log-evidence) must equal the library's own fused
filter run (vsmc_cuda_pf_run) with the same seed, and track the oracle's
FP32 filter."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from conftest import P, ROOT
from oracle.binding import ref_root

pytestmark = pytest.mark.gpu

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
REF = ref_root()


def build_sampler_program(out_path):
    """nvcc build of tests/cpp/sampler_cuda.cu against the reference tree;
    returns the binary's path."""
    from vsmc_gb300 import build
    lib = build.build()
    libdir = os.path.dirname(lib)
    cmd = [NVCC, "-std=c++17", "-O3", "-gencode",
           "arch=compute_103a,code=sm_103a",
           "-I", os.path.join(REF, "include"),
           "-I", os.path.join(ROOT, "tests", "cpp", "shim"),
           "-I", os.path.join(ROOT, "include"),
           "-DVSMC_RNG_TYPE=::vsmc::Philox4x32", "-DVSMC_HAS_MKL=0",
           "-DVSMC_HAS_TBB=0", "-Xcompiler", "-w"]
    if os.uname().machine == "aarch64":
        # the reference's SIMD header is x86-only (its include guard skips it)
        cmd += ["-DVSMC_UTILITY_SIMD_HPP", "-DVSMC_HAS_SSE2=0",
                "-DVSMC_HAS_AVX2=0", "-DVSMC_HAS_AES_NI=0",
                "-DVSMC_HAS_RDRAND=0"]
    cmd += [os.path.join(ROOT, "tests", "cpp", "sampler_cuda.cu"),
            "-o", str(out_path), "-L", libdir, "-lvsmc_cuda",
            f"-Xlinker=-rpath={libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stderr[-4000:])
    return str(out_path)


def run_sampler_program(exe, tmpdir, n, T, seed, scheme, threshold, dev_thr,
                        obs, runs=1, graph=True):
    """Runs the program; returns (histories, its JSON timing line).  graph:
    steps replayed as CUDA graphs (StateCUDA::use_graph)."""
    import json
    obs_path = os.path.join(str(tmpdir), "obs.bin")
    out_path = os.path.join(str(tmpdir), "out.bin")
    np.ascontiguousarray(obs, dtype=np.float64).tofile(obs_path)
    r = subprocess.run([exe, str(n), str(T), str(seed), str(scheme),
                        repr(threshold), "1" if dev_thr else "0", obs_path,
                        out_path, str(runs), "1" if graph else "0"],
                       capture_output=True, text=True, timeout=600)
    if r.returncode != 0:
        raise RuntimeError(r.stderr[-3000:])
    v = np.fromfile(out_path, dtype=np.float64)
    hist = {"mean": v[:2 * T].reshape(T, 2), "ess": v[2 * T:3 * T],
            "resampled": v[3 * T:4 * T].astype(np.int32),
            "logz": v[4 * T:5 * T]}
    return hist, json.loads(r.stdout.strip().splitlines()[-1])


@pytest.fixture(scope="module")
def exe(vc, tmp_path_factory):
    if REF is None:
        pytest.skip("reference headers not present on this host")
    return build_sampler_program(
        tmp_path_factory.mktemp("sampler") / "sampler_cuda")


def _obs(port, T):
    from oracle.binding import default_model
    tr = np.zeros(4 * T)
    ob = np.zeros(2 * T)
    port.vo_pf_simulate(0, T, ctypes.byref(default_model()), P(tr), P(ob))
    return ob.reshape(T, 2)


@pytest.mark.parametrize("scheme", [1, 2])
@pytest.mark.parametrize("dev_thr", [False, True])
def test_sampler_matches_fused_filter(vc, port, exe, tmp_path, scheme,
                                      dev_thr):
    n, T, seed, thr = 1 << 16, 80, 7, 0.5
    obs = _obs(port, T)
    got, _ = run_sampler_program(exe, tmp_path, n, T, seed, scheme, thr,
                                 dev_thr, obs)
    pf = vc.ParticleFilter(n, 32, scheme, thr, seed=seed, max_steps=T)
    want = pf.run(obs)
    pf.close()
    assert got["resampled"].sum() > 5
    assert np.array_equal(got["resampled"], want["resampled"])
    np.testing.assert_allclose(got["ess"], want["ess"], rtol=1e-6)
    np.testing.assert_allclose(got["logz"], want["logz"], rtol=1e-6,
                               atol=1e-6)
    np.testing.assert_allclose(got["mean"], want["mean"], rtol=1e-5,
                               atol=1e-5)


def test_sampler_tracks_oracle_fp32_filter(vc, port, exe, tmp_path):
    """The Sampler-driven run against the oracle's FP32 filter (same
    particle streams, the oracle resampling on FP64 weights): step 0 to
    1e-5, and the whole run within Monte Carlo error of it."""
    from oracle.binding import default_model
    n, T, seed = 1 << 14, 40, 3
    obs = _obs(port, T)
    got, _ = run_sampler_program(exe, tmp_path, n, T, seed, 2, 0.5, True, obs)
    mean = np.zeros(2 * T)
    ess = np.zeros(T)
    res = np.zeros(T, np.int32)
    logz = np.zeros(T)
    ob = np.ascontiguousarray(obs.ravel())
    port.vo_pf_run(32, n, T, seed, 2, 0.5, ctypes.byref(default_model()),
                   P(ob), 0, P(mean), P(ess), P(res), P(logz))
    assert abs(got["ess"][0] - ess[0]) / ess[0] < 1e-5
    assert abs(got["logz"][0] - logz[0]) < 1e-5 * max(1, abs(logz[0]))
    assert np.abs(got["mean"] - mean.reshape(T, 2)).max() < 0.5
    assert abs(got["logz"][-1] - logz[-1]) < 2.0


@pytest.mark.parametrize("dev_thr", [False, True])
def test_sampler_graph_replay_equals_launches(vc, port, exe, tmp_path,
                                              dev_thr):
    """Steps replayed from the captured graphs (one per buffer parity, kept
    across Sampler::initialize) give the histories of steps launched one by
    one, bit for bit, over two runs of the same sampler."""
    n, T, seed, thr = 100003, 40, 11, 0.6
    obs = _obs(port, T)
    a, _ = run_sampler_program(exe, tmp_path, n, T, seed, 2, thr, dev_thr,
                               obs, runs=2, graph=True)
    b, _ = run_sampler_program(exe, tmp_path, n, T, seed, 2, thr, dev_thr,
                               obs, runs=2, graph=False)
    assert a["resampled"].sum() > 3
    for k in ("mean", "ess", "resampled", "logz"):
        assert np.array_equal(a[k], b[k]), k
