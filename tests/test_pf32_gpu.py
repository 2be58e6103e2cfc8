"""FP32 / FP64 move + likelihood kernels, the simulator, and the FP32 fused
filter against the oracle."""
import ctypes

import numpy as np
import pytest

from conftest import P, dev, host, normal_pair_f64, particle_words

pytestmark = pytest.mark.gpu


def _model(vc):
    return vc.default_model()


def _omodel():
    from oracle.binding import default_model
    return default_model()


@pytest.mark.parametrize("t", [0, 1, 7])
@pytest.mark.parametrize("n", [1, 3, 1000, 4097])
def test_cv_move_f32_matches_oracle(vc, port, t, n):
    rng = np.random.default_rng(t * 1000 + n)
    state = rng.normal(0, 2, (4, n)).astype(np.float32)
    obs = np.array([0.7, -1.3])
    ds = dev(state.copy())
    ll = dev(np.zeros(n, np.float32))
    m = _model(vc)
    vc.call("vsmc_cuda_cv_move_f32", n, t, 12345, ctypes.byref(m), P(obs),
            ds.data_ptr(), ll.data_ptr(), None)
    s_ref = state.copy()
    l_ref = np.zeros(n, np.float32)
    om = _omodel()
    if t == 0:
        port.vo_pf_init_f32(n, 12345, ctypes.byref(om), P(obs), P(s_ref),
                            P(l_ref))
    else:
        port.vo_pf_move_f32(n, t, 12345, ctypes.byref(om), P(obs), P(s_ref),
                            P(l_ref))
    got_s = host(ds)
    got_l = host(ll)
    # FP32 kernel vs FP32 restatement: 1e-5 relative (absolute below 1)
    np.testing.assert_allclose(got_s, s_ref, rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(got_l, l_ref, rtol=1e-5, atol=1e-4)


def _cv_f64(m, t, seed, state, obs):
    """The model's move and log-likelihood in float64 on the FP32 kernel's
    own inputs: its FP32 state, its Philox words (key {t, seed}, counter
    {1, i, 0, 0}) and its 24-bit uniforms (the FP32 Box-Muller's (0, 1]
    radius and [0, 1) angle).  The full Student-t density of both
    coordinates (example/pf/include/pf.hpp:81-93 with its constants)."""
    from math import lgamma
    n = state.shape[1]
    w0, w1, w2, w3 = particle_words(t, seed, n)
    x = state.astype(np.float64)
    if t == 0:
        z1, z2 = normal_pair_f64(w0, w1)
        z3, z4 = normal_pair_f64(w2, w3)
        x = np.stack([m.sd_pos0 * z1, m.sd_pos0 * z2, m.sd_vel0 * z3,
                      m.sd_vel0 * z4])
    else:
        z1, z2 = normal_pair_f64(w0, w1)
        ax, ay = m.sigma_a * z1, m.sigma_a * z2
        h = 0.5 * m.dt * m.dt
        x = np.stack([x[0] + m.dt * x[2] + h * ax, x[1] + m.dt * x[3] + h * ay,
                      x[2] + m.dt * ax, x[3] + m.dt * ay])
    nu, s = m.nu, m.obs_scale
    c = lgamma(0.5 * (nu + 1)) - lgamma(0.5 * nu) - 0.5 * np.log(nu * np.pi) \
        - np.log(s)
    qx = ((obs[0] - x[0]) / s) ** 2 / nu
    qy = ((obs[1] - x[1]) / s) ** 2 / nu
    ll = 2 * c - 0.5 * (nu + 1) * (np.log1p(qx) + np.log1p(qy))
    return x, ll


@pytest.mark.parametrize("t", [0, 1, 50])
def test_cv_move_f32_vs_fp64_on_same_uniforms(vc, t):
    """The FP32 move and log-likelihood kernel against the FP64 evaluation of
    the same model on identical inputs (same state, words and uniforms):
    every element of the moved state and of the log-likelihood within 1e-5
    relative (1e-5 absolute below magnitude 1), over 2^20 particles, so the
    rare radius uniforms next to 1 are among them."""
    n, seed = 1 << 20, 9
    rng = np.random.default_rng(t)
    state32 = rng.normal(0, 2, (4, n)).astype(np.float32)
    obs = np.array([1.5, 0.25])
    ds = dev(state32.copy())
    ll = dev(np.zeros(n, np.float32))
    m = _model(vc)
    vc.call("vsmc_cuda_cv_move_f32", n, t, seed, ctypes.byref(m), P(obs),
            ds.data_ptr(), ll.data_ptr(), None)
    x64, l64 = _cv_f64(m, t, seed, state32, obs)
    got = host(ds).astype(np.float64)
    err = np.abs(got - x64) / np.maximum(1.0, np.abs(x64))
    assert err.max() < 1e-5, (err.max(), np.unravel_index(err.argmax(),
                                                          err.shape))
    gl = host(ll).astype(np.float64)
    el = np.abs(gl - l64) / np.maximum(1.0, np.abs(l64))
    assert el.max() < 1e-5, (el.max(), el.argmax())


@pytest.mark.parametrize("t", [0, 1, 99])
@pytest.mark.parametrize("n", [1, 5, 3000])
def test_cv_move_f64_matches_oracle(vc, port, t, n):
    rng = np.random.default_rng(t + 17 * n)
    state = rng.normal(0, 2, (4, n))
    obs = np.array([-0.3, 2.2])
    ds = dev(state.copy())
    ll = dev(np.zeros(n))
    m = _model(vc)
    vc.call("vsmc_cuda_cv_move_f64", n, t, 77, ctypes.byref(m), P(obs),
            ds.data_ptr(), ll.data_ptr(), None)
    s_ref = state.copy()
    l_ref = np.zeros(n)
    om = _omodel()
    if t == 0:
        port.vo_pf_init_f64(n, 77, ctypes.byref(om), P(obs), P(s_ref),
                            P(l_ref))
    else:
        port.vo_pf_move_f64(n, t, 77, ctypes.byref(om), P(obs), P(s_ref),
                            P(l_ref))
    np.testing.assert_allclose(host(ds), s_ref, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(host(ll), l_ref, rtol=1e-12, atol=1e-12)


def test_simulate_matches_oracle(vc, port):
    import torch
    T = 200
    truth = torch.zeros(4 * T, dtype=torch.float64, device="cuda")
    obs = torch.zeros(2 * T, dtype=torch.float64, device="cuda")
    m = _model(vc)
    vc.call("vsmc_cuda_cv_simulate", 0, T, ctypes.byref(m), truth.data_ptr(),
            obs.data_ptr(), None)
    tr = np.zeros(4 * T)
    ob = np.zeros(2 * T)
    port.vo_pf_simulate(0, T, ctypes.byref(_omodel()), P(tr), P(ob))
    np.testing.assert_allclose(host(truth), tr, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(host(obs), ob, rtol=1e-12, atol=1e-12)


def _obs(port, T=100, seed=0):
    tr = np.zeros(4 * T)
    ob = np.zeros(2 * T)
    port.vo_pf_simulate(seed, T, ctypes.byref(_omodel()), P(tr), P(ob))
    return ob.reshape(T, 2), tr.reshape(T, 4)


def _oracle_pf(port, prec, n, T, seed, scheme, obs):
    mean = np.zeros(2 * T)
    ess = np.zeros(T)
    res = np.zeros(T, np.int32)
    logz = np.zeros(T)
    port.vo_pf_run(prec, n, T, seed, scheme, 0.5, ctypes.byref(_omodel()),
                   P(np.ascontiguousarray(obs)), 0, P(mean), P(ess), P(res),
                   P(logz))
    return {"mean": mean.reshape(T, 2), "ess": ess, "resampled": res,
            "logz": logz}


@pytest.mark.parametrize("scheme", [1, 2])
@pytest.mark.parametrize("graph", [True, False])
def test_pf32_filter_tracks_oracle(vc, port, scheme, graph):
    """Same particle streams and resampling engine as the oracle's FP32
    filter; the CDFs differ (fixed-point vs left-to-right FP64), so compare
    with tolerances well inside the Monte Carlo error."""
    T, n = 100, 1 << 14
    obs, truth = _obs(port, T)
    pf = vc.ParticleFilter(n, 32, scheme, 0.5, seed=3, max_steps=T)
    pf.use_graph(graph)
    g = pf.run(obs)
    pf.close()
    o = _oracle_pf(port, 32, n, T, 3, scheme, obs)
    # step 0 is identical up to FP32 rounding
    assert abs(g["ess"][0] - o["ess"][0]) / o["ess"][0] < 1e-4
    assert abs(g["logz"][0] - o["logz"][0]) < 1e-4
    # whole run: means and evidence within Monte Carlo error
    assert np.abs(g["mean"] - o["mean"]).max() < 0.2
    assert abs(g["logz"][-1] - o["logz"][-1]) < 1.0
    assert np.abs(g["mean"] - truth[:, :2]).mean() < 0.5
    assert g["resampled"].sum() > 5


def _download_i32(dev_ptr, count):
    """count int32 values from a raw device address (through torch)."""
    import torch
    out = torch.empty(count, dtype=torch.int32, device="cuda")
    cudart = None
    for name in ("libcudart.so.13", "libcudart.so"):
        try:
            cudart = ctypes.CDLL(name)
            break
        except OSError:
            continue
    assert cudart is not None
    torch.cuda.synchronize()
    rc = cudart.cudaMemcpy(ctypes.c_void_p(out.data_ptr()),
                           ctypes.c_void_p(dev_ptr), ctypes.c_size_t(4 * count),
                           ctypes.c_int(3))  # device to device
    assert rc == 0, rc
    return out.cpu().numpy()


@pytest.mark.parametrize("scheme", [1, 2])
def test_pf32_filter_every_step_against_oracle_replay(vc, port, scheme):
    """The whole run, step by step: the oracle's FP32 filter replays the
    device's own resampling (its decisions and genealogy rows), so the two
    runs hold the same particles at every step and differ only by FP32
    rounding in the move, the weights and the reductions.  Every step's ESS,
    log-evidence and filtering mean must agree tightly, and every device
    decision must match the oracle's ESS against the threshold unless the
    ESS sits within 1e-4 of it."""
    T, n = 100, 1 << 14
    obs, _ = _obs(port, T)
    pf = vc.ParticleFilter(n, 32, scheme, 0.5, seed=3, max_steps=T)
    pf.record_genealogy(True)
    g = pf.run(obs)
    rows = _download_i32(pf.genealogy_ptr(), T * n)
    pf.close()
    mean = np.zeros(2 * T)
    ess = np.zeros(T)
    logz = np.zeros(T)
    res = np.ascontiguousarray(g["resampled"], np.int32)
    port.vo_pf_run_replay(32, n, T, 3, ctypes.byref(_omodel()),
                          P(np.ascontiguousarray(obs)), P(res), P(rows),
                          P(mean), P(ess), P(logz))
    mean = mean.reshape(T, 2)
    assert res.sum() > 5
    rel_ess = np.abs(g["ess"] - ess) / ess
    assert rel_ess.max() < 1e-4, (rel_ess.argmax(), rel_ess.max())
    assert np.abs(g["logz"] - logz).max() < 1e-3, np.abs(g["logz"] - logz).max()
    assert np.abs(g["mean"] - mean).max() < 1e-3, np.abs(g["mean"] - mean).max()
    near = np.abs(ess / n - 0.5) < 1e-4
    decided = (ess < 0.5 * n).astype(np.int32)
    assert np.array_equal(res[~near], decided[~near])


def test_pf32_reproducible_and_graph_equal(vc, port):
    T, n = 60, 50000
    obs, _ = _obs(port, T, seed=4)
    outs = []
    for graph in (True, False, True):
        pf = vc.ParticleFilter(n, 32, 2, 0.5, seed=8, max_steps=T)
        pf.use_graph(graph)
        outs.append(pf.run(obs))
        pf.close()
    for o in outs[1:]:
        for k in ("mean", "ess", "resampled", "logz"):
            assert np.array_equal(o[k], outs[0][k]), k


@pytest.mark.parametrize("n", [2, 3, 5, 1000, 4097])
def test_pf32_filter_small_and_ragged_sizes(vc, port, n):
    """Particle counts below one 4-particle group, below one tile and just
    above a tile: the run completes with finite histories, every ESS lies in
    [1, n], and step 0 (same streams, no resampling yet) matches the
    oracle's FP32 filter up to FP32 rounding."""
    T = 20
    obs, _ = _obs(port, T, seed=6)
    pf = vc.ParticleFilter(n, 32, 1, 0.5, seed=2, max_steps=T)
    g = pf.run(obs)
    pf.close()
    for k in ("mean", "ess", "logz"):
        assert np.isfinite(g[k]).all(), k
    assert (g["ess"] >= 1 - 1e-6).all() and (g["ess"] <= n + 1e-6).all()
    o = _oracle_pf(port, 32, n, T, 2, 1, obs)
    assert abs(g["ess"][0] - o["ess"][0]) / o["ess"][0] < 1e-4
    assert abs(g["logz"][0] - o["logz"][0]) < 1e-4
    assert g["resampled"][0] == o["resampled"][0]


def test_pf32_filter_at_2_to_28_particles(vc, port):
    """N = 2^28 (about 14 GB of state, weights and resampling arrays): the
    32-bit particle indices, the 35-bit fixed-point CDF and the 128-bit
    position arithmetic at scale.  The run must agree with an N = 2^20 run
    of the same model and observations within Monte Carlo error (the
    smaller run's error dominates), and resample at step 0 like it."""
    T = 4
    obs, _ = _obs(port, T, seed=9)
    out = {}
    for lg in (20, 28):
        pf = vc.ParticleFilter(1 << lg, 32, 2, 0.5, seed=4, max_steps=T)
        out[lg] = pf.run(obs)
        pf.close()
    big, small = out[28], out[20]
    for k in ("mean", "ess", "logz"):
        assert np.isfinite(big[k]).all(), k
    assert big["resampled"][0] == small["resampled"][0] == 1
    np.testing.assert_allclose(big["ess"][0] / 2 ** 28,
                               small["ess"][0] / 2 ** 20, rtol=0.02)
    assert np.abs(big["logz"] - small["logz"]).max() < 0.05
    assert np.abs(big["mean"] - small["mean"]).max() < 0.05
