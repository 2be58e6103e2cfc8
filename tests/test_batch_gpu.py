"""Batched FP32 filters (vsmc_cuda_batch) against single filters with the
same seeds and models, against each other across kernel shapes, and a
default-model member against the oracle's FP32 filter."""
import ctypes

import numpy as np
import pytest

from conftest import P, dev, host

pytestmark = pytest.mark.gpu


def _spec(vc, nf=24, seed=0, nmax_log2=15, tmax=80):
    rng = np.random.default_rng(seed)
    n = np.exp(rng.uniform(np.log(2), np.log(2 ** nmax_log2), nf)).astype(
        np.uint32)
    n[:4] = [2, 3, 5, 4097][:min(4, nf)]
    T = rng.integers(1, tmax + 1, nf).astype(np.uint32)
    T[0] = 1
    seeds = (1000 + np.arange(nf)).astype(np.uint32)
    models = []
    for f in range(nf):
        m = vc.default_model()
        m.sigma_a = float(rng.uniform(0.5, 2.0))
        m.obs_scale = float(rng.uniform(0.2, 1.0))
        models.append(m)
    return n, T, seeds, models


def _simulate(vc, batch):
    import torch
    obs = torch.zeros(2 * batch.total_steps, dtype=torch.float64,
                      device="cuda")
    batch.simulate(obs.data_ptr())
    return obs


def test_batch_simulate_matches_single_simulator(vc):
    import torch
    n, T, seeds, models = _spec(vc, nf=9)
    b = vc.FilterBatch(n, T, seeds, models)
    obs = host(_simulate(vc, b)).reshape(-1, 2)
    for f in range(len(n)):
        tr = torch.zeros(4 * int(T[f]), dtype=torch.float64, device="cuda")
        ob = torch.zeros(2 * int(T[f]), dtype=torch.float64, device="cuda")
        vc.call("vsmc_cuda_cv_simulate", int(seeds[f]), int(T[f]),
                ctypes.byref(models[f]), tr.data_ptr(), ob.data_ptr(), None)
        a, z = int(b.offsets[f]), int(b.offsets[f + 1])
        assert np.array_equal(obs[a:z], host(ob).reshape(-1, 2)), f
    b.close()


def _spec_config4(vc, nf, seed):
    """Filters drawn like the benchmark's batch: particles log-uniform in
    [2^8, 2^16], horizons uniform in [50, 500], sigma_a U(0.5, 2), obs
    scale U(0.2, 1)."""
    rng = np.random.default_rng(100 + seed)
    n = np.exp(rng.uniform(np.log(2 ** 8), np.log(2 ** 16), nf)).astype(
        np.uint32)
    n[0] = 1 << 16
    T = rng.integers(50, 501, nf).astype(np.uint32)
    T[0] = 500
    seeds = (5000 + np.arange(nf)).astype(np.uint32)
    models = []
    for f in range(nf):
        m = vc.default_model()
        m.sigma_a = float(rng.uniform(0.5, 2.0))
        m.obs_scale = float(rng.uniform(0.2, 1.0))
        models.append(m)
    return n, T, seeds, models


@pytest.mark.parametrize("size", ["small", "config4"])
@pytest.mark.parametrize("scheme", [1, 2])
def test_batch_members_match_single_filters(vc, scheme, size):
    """Filter f of the batch against vsmc_cuda_pf with seed f and model f:
    identical particles and counts, so identical resampling decisions; the
    FP64 sums differ only in their order.  The single filter is checked
    step by step against the oracle (test_pf32_gpu.py), so this carries the
    oracle's parity to every member, at the benchmark batch's sizes too
    (up to 2^16 particles and 500 steps)."""
    if size == "small":
        n, T, seeds, models = _spec(vc, nf=24, seed=scheme)
    else:
        n, T, seeds, models = _spec_config4(vc, nf=48, seed=scheme)
    b = vc.FilterBatch(n, T, seeds, models, scheme=scheme)
    obs = host(_simulate(vc, b)).reshape(-1, 2)
    got = b.run(obs)
    b.close()
    for f in range(len(n)):
        a, z = int(b.offsets[f]), int(b.offsets[f + 1])
        pf = vc.ParticleFilter(int(n[f]), 32, scheme, 0.5, seed=int(seeds[f]),
                               model=models[f], max_steps=int(T[f]))
        ref = pf.run(obs[a:z])
        pf.close()
        g = got[f]
        assert np.array_equal(g["resampled"], ref["resampled"]), f
        np.testing.assert_allclose(g["ess"], ref["ess"], rtol=1e-9)
        np.testing.assert_allclose(g["logz"], ref["logz"], rtol=1e-9,
                                   atol=1e-9)
        np.testing.assert_allclose(g["mean"], ref["mean"], rtol=1e-5,
                                   atol=1e-5)


def test_batch_shapes_agree_and_autotune(vc):
    import torch
    n, T, seeds, models = _spec(vc, nf=40, seed=7, nmax_log2=14, tmax=40)
    b = vc.FilterBatch(n, T, seeds, models)
    obs = _simulate(vc, b)
    outs = []
    for ppt, block in [(1, 128), (2, 128), (4, 128), (1, 256), (2, 256),
                       (4, 256)]:
        b.set_shape(ppt, block)
        assert b.shape() == (ppt, block)
        b.run_device(obs.data_ptr())
        outs.append(b.history())
    for o in outs[1:]:
        for f in range(len(n)):
            assert np.array_equal(o[f]["resampled"], outs[0][f]["resampled"])
            # the shape changes how FP32 partial sums are grouped
            np.testing.assert_allclose(o[f]["logz"], outs[0][f]["logz"],
                                       rtol=1e-7, atol=1e-7)
            np.testing.assert_allclose(o[f]["mean"], outs[0][f]["mean"],
                                       rtol=1e-5, atol=1e-5)
    ms = b.autotune(obs.data_ptr(), steps=20)
    assert (ms > 0).all()
    assert b.shape() in [(1, 128), (2, 128), (4, 128), (1, 256), (2, 256),
                         (4, 256)]
    b.run_device(obs.data_ptr())
    after = b.history()
    for f in range(len(n)):
        assert np.array_equal(after[f]["resampled"], outs[0][f]["resampled"])
    b.close()


def test_batch_member_tracks_oracle(vc, port):
    """A default-model member against the oracle's FP32 filter (same
    streams; the CDFs differ, so within Monte Carlo error)."""
    from oracle.binding import default_model
    T, N = 100, 1 << 14
    tr = np.zeros(4 * T)
    ob = np.zeros(2 * T)
    port.vo_pf_simulate(0, T, ctypes.byref(default_model()), P(tr), P(ob))
    b = vc.FilterBatch([N, 300], [T, 20], [3, 4])
    obs = np.concatenate([ob.reshape(T, 2), ob.reshape(T, 2)[:20]])
    g = b.run(obs)[0]
    b.close()
    mean = np.zeros(2 * T)
    ess = np.zeros(T)
    res = np.zeros(T, np.int32)
    logz = np.zeros(T)
    port.vo_pf_run(32, N, T, 3, 1, 0.5, ctypes.byref(default_model()), P(ob),
                   0, P(mean), P(ess), P(res), P(logz))
    assert abs(g["ess"][0] - ess[0]) / ess[0] < 1e-4
    assert abs(g["logz"][0] - logz[0]) < 1e-4
    assert np.abs(g["mean"] - mean.reshape(T, 2)).max() < 0.2
    assert abs(g["logz"][-1] - logz[-1]) < 1.0
    assert np.abs(g["mean"] - tr.reshape(T, 4)[:, :2]).mean() < 0.5


def test_batch_scan_schedules_agree_and_autotune(vc):
    """The resampling chunk (scan schedule) changes how a filter's particles
    are split across the list, not the counts: every schedule gives the same
    histories, bit for bit, and the schedule autotuner keeps one of them."""
    n, T, seeds, models = _spec(vc, nf=40, seed=11, nmax_log2=16, tmax=60)
    b = vc.FilterBatch(n, T, seeds, models)
    obs = _simulate(vc, b)
    outs = []
    for c in (4096, 8192, 16384, 32768):
        b.set_schedule(c)
        assert b.schedule() == c
        b.run_device(obs.data_ptr())
        outs.append(b.history())
    for o in outs[1:]:
        for f in range(len(n)):
            for k in ("mean", "ess", "resampled", "logz"):
                assert np.array_equal(o[f][k], outs[0][f][k]), (f, k)
    with pytest.raises(vc.VsmcCudaError):
        b.set_schedule(5000)
    ms = b.autotune_schedule(obs.data_ptr(), steps=20)
    assert (ms > 0).all()
    assert b.schedule() in (4096, 8192, 16384, 32768)
    b.close()
