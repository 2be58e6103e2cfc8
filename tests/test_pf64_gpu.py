"""FP64 filter with the reference's arithmetic vs the oracle filter."""
import ctypes

import numpy as np
import pytest

from conftest import P

pytestmark = pytest.mark.gpu


def _obs(port, T, seed=0):
    from oracle.binding import default_model
    tr = np.zeros(4 * T)
    ob = np.zeros(2 * T)
    port.vo_pf_simulate(seed, T, ctypes.byref(default_model()), P(tr), P(ob))
    return ob.reshape(T, 2)


def _oracle(port, n, T, seed, scheme, obs, prec=64):
    from oracle.binding import default_model
    mean = np.zeros(2 * T)
    ess = np.zeros(T)
    res = np.zeros(T, np.int32)
    logz = np.zeros(T)
    port.vo_pf_run(prec, n, T, seed, scheme, 0.5,
                   ctypes.byref(default_model()), P(np.ascontiguousarray(obs)),
                   0, P(mean), P(ess), P(res), P(logz))
    return {"mean": mean.reshape(T, 2), "ess": ess, "resampled": res,
            "logz": logz}


@pytest.mark.parametrize("scheme", range(6))
def test_pf64_tracks_oracle(vc, port, scheme):
    T, n = 100, 1 << 14
    obs = _obs(port, T)
    pf = vc.ParticleFilter(n, 64, scheme, 0.5, seed=5, max_steps=T)
    g = pf.run(obs)
    pf.close()
    o = _oracle(port, n, T, 5, scheme, obs)
    assert np.array_equal(g["resampled"], o["resampled"])
    np.testing.assert_allclose(g["ess"], o["ess"], rtol=1e-8)
    np.testing.assert_allclose(g["mean"], o["mean"], rtol=1e-8, atol=1e-8)
    np.testing.assert_allclose(g["logz"], o["logz"], rtol=1e-9, atol=1e-8)


def test_pf64_iterate_equals_run(vc, port):
    import torch
    T, n = 30, 4096
    obs = _obs(port, T, seed=2)
    pf = vc.ParticleFilter(n, 64, 1, 0.5, seed=1, max_steps=T)
    g = pf.run(obs)
    pf.close()
    pf = vc.ParticleFilter(n, 64, 1, 0.5, seed=1, max_steps=T)
    d = torch.from_numpy(obs.copy()).cuda()
    vc.call("vsmc_cuda_pf_initialize", pf.handle, d[0].data_ptr())
    for t in range(1, T):
        vc.call("vsmc_cuda_pf_iterate", pf.handle, d[t].data_ptr())
    h = pf.history(T)
    pf.close()
    for k in ("mean", "ess", "resampled", "logz"):
        assert np.array_equal(g[k], h[k]), k
