"""Resample-move: the kernel-level random-walk Metropolis step against the
oracle, and the FP32 filter with MCMC sweeps after resampling."""
import ctypes

import numpy as np
import pytest

from conftest import P, dev, host

pytestmark = pytest.mark.gpu


def _omodel():
    from oracle.binding import default_model
    return default_model()


@pytest.mark.parametrize("parent", [False, True])
def test_cv_mcmc_matches_oracle(vc, port, parent):
    import torch
    n, t, sweeps, scale = 4000, 3, 5, 0.7
    rng = np.random.default_rng(2 + parent)
    state = rng.normal(0, 1.5, (4, n)).astype(np.float32)
    obs = np.array([0.3, -0.4])
    par = np.sort(rng.integers(0, n, n)).astype(np.int32) if parent else None
    ds = dev(state.copy())
    acc = torch.zeros(1, dtype=torch.int32, device="cuda")
    m = vc.default_model()
    vc.call("vsmc_cuda_cv_mcmc_f32", n, t, sweeps, 21, ctypes.byref(m),
            P(obs), scale, dev(par).data_ptr() if parent else None,
            ds.data_ptr(), acc.data_ptr(), None)
    ref = state.copy()
    racc = ctypes.c_uint32(0)
    margin = np.zeros(n, np.float32)
    port.vo_cv_mcmc_f32(n, t, sweeps, 21, ctypes.byref(_omodel()), P(obs),
                        scale, P(par) if parent else None, P(ref),
                        ctypes.byref(racc), P(margin))
    got = host(ds)
    # An accept decision whose log-uniform lies within FP32 rounding of the
    # log acceptance ratio can go the other way (the device's normal pair
    # and log-density use the SFU).  Every particle that differs must have
    # had such a decision on the oracle's path: its closest |log u - log
    # ratio| over the sweeps is below 1e-4 (typical values are O(1)).
    bad = ~np.isclose(got, ref, rtol=1e-4, atol=1e-4).all(axis=0)
    unexplained = bad & (margin >= 1e-4)
    assert not unexplained.any(), (np.flatnonzero(unexplained)[:10],
                                   margin[unexplained][:10])
    assert bad.mean() < 5e-3, bad.mean()
    a = int(host(acc)[0])
    assert abs(a - racc.value) <= max(5, 0.005 * racc.value)
    assert 0.05 * n * sweeps < a < 0.95 * n * sweeps


def _obs(port, T, seed):
    tr = np.zeros(4 * T)
    ob = np.zeros(2 * T)
    port.vo_pf_simulate(seed, T, ctypes.byref(_omodel()), P(tr), P(ob))
    return ob.reshape(T, 2), tr.reshape(T, 4)


def test_filter_resample_move(vc, port):
    T, n = 60, 1 << 14
    obs, truth = _obs(port, T, 6)
    outs = {}
    for sweeps in (0, 3):
        for graph in (True, False):
            pf = vc.ParticleFilter(n, 32, 1, 0.5, seed=9, max_steps=T)
            pf.set_mcmc(sweeps, 0.5)
            pf.use_graph(graph)
            g = pf.run(obs)
            g["acc"] = pf.mcmc_accepts(T) if sweeps else None
            g["tsv"] = pf.print_tsv(T)
            pf.close()
            outs[(sweeps, graph)] = g
    plain, move = outs[(0, True)], outs[(3, True)]
    # graph and stream launches agree
    for k in ("mean", "ess", "resampled", "logz"):
        assert np.array_equal(outs[(3, False)][k], move[k]), k
    # accepts only after resampling steps (t >= 1)
    res = move["resampled"].astype(bool)
    acc = move["acc"]
    assert (acc[~res] == 0).all() and acc[0] == 0
    rate = acc[1:][res[1:]] / (3.0 * n)
    assert (rate > 0.05).all() and (rate < 0.95).all()
    # same posterior: means and evidence within Monte Carlo error
    assert np.abs(move["mean"] - plain["mean"]).max() < 0.25
    assert abs(move["logz"][-1] - plain["logz"][-1]) < 1.5
    assert np.abs(move["mean"] - truth[:, :2]).mean() < 0.5
    # the summary text carries the MCMC accept column
    head = move["tsv"].splitlines()[0].split("\t")
    assert head[:5] == ["Size", "Resampled", "Accept.0", "Accept.1", "ESS"]
    row = move["tsv"].splitlines()[2].split("\t")
    assert int(row[3]) == int(acc[1])
