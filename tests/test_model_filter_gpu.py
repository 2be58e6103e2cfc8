"""User device models through the fused FP32 filter (the MoveCUDA hook).

tests/cpp/model_filter.cu instantiates the public step-kernel template of
include/vsmc_cuda_filter.cuh with models written in test code, and drives
the filter through the C ABI (vsmc_cuda_pf_create_model, _step_desc_get,
_step_commit, _resample_now, _get_status): the device-side twin of
MoveBase::eval_sp under MoveOMP::operator() (smp/backend_base.hpp:243-363,
smp/backend_omp.hpp:93-105) with Particle::resample deciding on the host
(core/particle.hpp:170-197).

* The constant-velocity model written as user code gives the built-in
  filter's histories: same resampling decisions, ESS, log-evidence and
  monitor, whether the device or the host takes the resampling decision.
* A 2-D random walk (dim 2, one monitored component) matches a float64
  numpy restatement over the same Philox words (FP32 tolerance, 2e-4).
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from conftest import P, ROOT, normal_pair_f64, philox4x32_10

pytestmark = pytest.mark.gpu

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")


@pytest.fixture(scope="module")
def mf(vc, tmp_path_factory):
    from vsmc_gb300 import build
    lib = build.build()
    out = tmp_path_factory.mktemp("model_filter") / "libmodel_filter.so"
    libdir = os.path.dirname(lib)
    cmd = [NVCC, "-std=c++17", "-O3", "-gencode",
           "arch=compute_103a,code=sm_103a", "-Xcompiler", "-fPIC",
           "-shared", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "model_filter.cu"),
           "-o", str(out), "-L", libdir, "-lvsmc_cuda",
           f"-Xlinker=-rpath={libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    L = ctypes.CDLL(str(out))
    L.model_filter_run.restype = ctypes.c_int
    L.model_filter_run.argtypes = [ctypes.c_int, ctypes.c_void_p,
                                   ctypes.c_size_t, ctypes.c_size_t,
                                   ctypes.c_uint32, ctypes.c_int,
                                   ctypes.c_double, ctypes.c_int,
                                   ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_void_p]
    return L


def _run(mf, model, p, n, T, seed, scheme, threshold, host, obs, mdim):
    obs = np.ascontiguousarray(obs, dtype=np.float64)
    mean = np.zeros((T, mdim))
    ess = np.zeros(T)
    res = np.zeros(T, np.int32)
    logz = np.zeros(T)
    pv = np.ascontiguousarray(p, dtype=np.float64)
    rc = mf.model_filter_run(model, P(pv), n, T, seed, scheme, threshold,
                             1 if host else 0, P(obs), P(mean), P(ess),
                             P(res), P(logz))
    assert rc == 0, rc
    return {"mean": mean, "ess": ess, "resampled": res, "logz": logz}


def _cv_obs(port, T):
    from oracle.binding import default_model
    tr = np.zeros(4 * T)
    ob = np.zeros(2 * T)
    port.vo_pf_simulate(0, T, ctypes.byref(default_model()), P(tr), P(ob))
    return ob.reshape(T, 2)


@pytest.mark.parametrize("scheme", [1, 2])
@pytest.mark.parametrize("host", [False, True])
@pytest.mark.parametrize("n", [(1 << 16) + 3, 5000])
def test_user_cv_model_matches_builtin_filter(vc, port, mf, scheme, host, n):
    T, seed, thr = 60, 11, 0.5
    obs = _cv_obs(port, T)
    m = vc.default_model()
    p = [m.dt, m.sigma_a, m.obs_scale, m.nu, m.sd_pos0, m.sd_vel0]
    got = _run(mf, 0, p, n, T, seed, scheme, thr, host, obs, 2)
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


# ---------------------------------------------------------------- walk2

def test_walk2_model_matches_numpy_restatement(mf):
    n, T, seed = 4096, 6, 3
    sd0, s, r = 1.5, 0.7, 0.9
    rng = np.random.default_rng(5)
    obs = rng.normal(0, 2, (T, 2))
    # threshold 0: ESS < 0 never holds, so the weights accumulate
    got = _run(mf, 1, [sd0, s, r], n, T, seed, 2, 0.0, False, obs, 1)
    i = np.arange(n, dtype=np.uint64)
    x = np.zeros((2, n))
    lw = np.zeros(n)
    logz = 0.0
    lconst = -np.log(2 * np.pi) - 2 * np.log(r)
    for t in range(T):
        w0, w1, _, _ = philox4x32_10([np.ones(n, np.uint64), i,
                                      np.zeros(n, np.uint64),
                                      np.zeros(n, np.uint64)], t, seed)
        a, b = normal_pair_f64(w0, w1)
        if t == 0:
            x = np.stack([sd0 * a, sd0 * b])
        else:
            x = x + s * np.stack([a, b])
        ll = lconst - 0.5 * (((obs[t, 0] - x[0]) / r) ** 2 +
                             ((obs[t, 1] - x[1]) / r) ** 2)
        prev = lw - lw.max()
        W = np.exp(prev) / np.exp(prev).sum()
        logz += np.log(np.sum(W * np.exp(ll)))
        lw = lw + ll
        e = np.exp(lw - lw.max())
        ess = e.sum() ** 2 / (e * e).sum()
        mean0 = np.sum(e * x[0]) / e.sum()
        assert got["resampled"][t] == 0
        assert abs(got["ess"][t] - ess) / ess < 2e-4, (t, got["ess"][t], ess)
        assert abs(got["logz"][t] - logz) < 2e-4 * max(1.0, abs(logz)), t
        assert abs(got["mean"][t, 0] - mean0) < 2e-4 * max(1.0, abs(mean0)), t


def test_walk2_resampling_keeps_mass(mf):
    """Host-decided resampling every step (threshold 2: ESS < 2N always):
    the log-evidence stays finite and every step reports a resample."""
    n, T = 3000, 20
    obs = np.random.default_rng(9).normal(0, 1, (T, 2))
    got = _run(mf, 1, [1.0, 0.5, 0.8], n, T, 4, 1, 2.0, True, obs, 1)
    assert got["resampled"].tolist() == [1] * T
    assert np.all(np.isfinite(got["logz"]))
    assert np.all(got["ess"] > 0) and np.all(got["ess"] <= n * (1 + 1e-9))
