"""Learned proposal (bearings-only model): the device simulator, network
forward pass, loss gradient and per-particle move / weight against the
oracle (which reproduces the device's BF16 operand rounding); the batched
bootstrap and learned filters against the oracle's filters; and training
that lowers the spread of the log-evidence estimate."""
import ctypes

import numpy as np
import pytest

from conftest import P, dev, host

pytestmark = pytest.mark.gpu

NPAR = 64 * 6 + 64 + 64 * 64 + 64 + 8 * 64 + 8


def _omodel():
    from oracle.binding import bearings_model
    return bearings_model()


def _params(rng, out_scale=0.3):
    p = rng.normal(0, 0.3, NPAR).astype(np.float32)
    p[4544:4544 + 8 * 64] *= out_scale / 0.3  # W3
    return p


def _pack(vc, p):
    import torch
    prop = vc.Proposal()
    prop.params.copy_(torch.from_numpy(p).cuda())
    prop.pack()
    return prop


def test_bearings_simulate_matches_oracle(vc, port):
    import torch
    T = 200
    truth = torch.zeros(4 * T, dtype=torch.float64, device="cuda")
    obs = torch.zeros(T, dtype=torch.float64, device="cuda")
    m = vc.bearings_model()
    vc.call("vsmc_cuda_bearings_simulate", 0, T, ctypes.byref(m),
            truth.data_ptr(), obs.data_ptr(), None)
    tr = np.zeros(4 * T)
    ob = np.zeros(T)
    port.vo_bearings_simulate(0, T, ctypes.byref(_omodel()), P(tr), P(ob))
    np.testing.assert_allclose(host(truth), tr, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(host(obs), ob, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("B", [1, 17, 1000])
def test_mlp_forward_matches_oracle(vc, port, B):
    import torch
    rng = np.random.default_rng(B)
    p = _params(rng)
    prop = _pack(vc, p)
    feat = rng.normal(0, 1, (B, 6)).astype(np.float32)
    out = torch.zeros((B, 8), dtype=torch.float32, device="cuda")
    vc.call("vsmc_cuda_mlp_forward", prop.packed.data_ptr(), B,
            dev(feat).data_ptr(), out.data_ptr(), None)
    ref = np.zeros((B, 8), np.float32)
    port.vo_mlp_forward(P(p), B, P(feat), P(ref))
    err = np.abs(host(out) - ref) / (1 + np.abs(ref))
    # FP32 vs FP64 sums; an activation that lands on a BF16 rounding
    # boundary can round the other way
    assert np.quantile(err, 0.99) < 1e-4
    assert err.max() < 1e-2


@pytest.mark.parametrize("B", [1, 17, 1000, 40000])
def test_mlp_forward_tc_matches_oracle(vc, port, B):
    """The tcgen05 form of the network (128 rows per tile) against the
    oracle, and against the mma.sync form on the same inputs."""
    import torch
    rng = np.random.default_rng(B + 1)
    p = _params(rng)
    prop = _pack(vc, p)
    feat = rng.normal(0, 1, (B, 6)).astype(np.float32)
    out = torch.zeros((B, 8), dtype=torch.float32, device="cuda")
    out_ms = torch.zeros((B, 8), dtype=torch.float32, device="cuda")
    df = dev(feat)
    vc.call("vsmc_cuda_mlp_forward_tc", prop.packed.data_ptr(), B,
            df.data_ptr(), out.data_ptr(), None)
    vc.call("vsmc_cuda_mlp_forward", prop.packed.data_ptr(), B,
            df.data_ptr(), out_ms.data_ptr(), None)
    ref = np.zeros((B, 8), np.float32)
    port.vo_mlp_forward(P(p), B, P(feat), P(ref))
    got = host(out)
    assert np.isfinite(got).all()
    # FP32 sums in another order than the oracle's and mma.sync's; an
    # activation on a BF16 rounding boundary can round the other way, which
    # moves that row's outputs by about one BF16 step of a hidden unit
    for other in (ref, host(out_ms)):
        err = np.abs(got - other) / (1 + np.abs(ref))
        assert np.quantile(err, 0.99) < 1e-4
        assert np.quantile(err, 0.9999) < 1e-2
        assert err.max() < 5e-2


@pytest.mark.parametrize("B", [1, 777, 65536])
def test_mlp_loss_grad_matches_oracle(vc, port, B):
    """B = 65536 gives every block of the tensor-core contraction several
    rounds, so both stage buffers are reused."""
    import torch
    rng = np.random.default_rng(5)
    p = _params(rng)
    prop = _pack(vc, p)
    feat = rng.normal(0, 1, (B, 6)).astype(np.float32)
    nu = rng.normal(0, 1, (B, 4)).astype(np.float32)
    loss = torch.zeros(1, dtype=torch.float64, device="cuda")
    grad = torch.zeros(NPAR, dtype=torch.float32, device="cuda")
    vc.call("vsmc_cuda_mlp_loss_grad", prop.packed.data_ptr(), B,
            dev(feat).data_ptr(), dev(nu).data_ptr(), loss.data_ptr(),
            grad.data_ptr(), None)
    rl = ctypes.c_double()
    rg = np.zeros(NPAR)
    port.vo_mlp_loss_grad(P(p), B, P(feat), P(nu), ctypes.byref(rl), P(rg))
    assert abs(host(loss)[0] - rl.value) <= 1e-5 * abs(rl.value)
    g = host(grad).astype(np.float64)
    rel = np.linalg.norm(g - rg) / np.linalg.norm(rg)
    assert rel < 2e-3, rel
    # every block of the parameter vector
    for a, b in ((0, 384), (384, 448), (448, 4544), (4544, 4608),
                 (4608, 5120), (5120, 5128)):
        r = np.linalg.norm(g[a:b] - rg[a:b]) / np.linalg.norm(rg[a:b])
        assert r < 5e-3, (a, b, r)


@pytest.mark.parametrize("t", [0, 3])
@pytest.mark.parametrize("learned", [False, True])
def test_bearings_move_matches_oracle(vc, port, t, learned):
    import torch
    n = 1000
    rng = np.random.default_rng(t + 10 * learned)
    state = np.stack([rng.normal(10, 1, n), rng.normal(10, 1, n),
                      rng.normal(0, 1, n), rng.normal(0, 1, n)]).astype(
                          np.float32)
    z = float(np.arctan2(10.3, 9.8))
    p = _params(rng, out_scale=0.05)
    prop = _pack(vc, p) if learned else None
    ds = dev(state.copy())
    lw = torch.zeros(n, dtype=torch.float32, device="cuda")
    m = vc.bearings_model()
    om = _omodel()
    if learned:
        # a wider bearing noise: the likelihood amplifies a position
        # difference d into (r / sigma_z) d on the normalised error, and
        # the check is on the move and the proposal term, not on that gain
        m.sigma_z = om.sigma_z = 0.05
    vc.call("vsmc_cuda_bearings_move_f32", n, t, 77, ctypes.byref(m), z,
            prop.packed.data_ptr() if learned else None, ds.data_ptr(),
            lw.data_ptr(), None)
    s_ref = state.copy()
    l_ref = np.zeros(n, np.float32)
    port.vo_bearings_move_f32(n, t, 77, ctypes.byref(om), z,
                              P(p) if learned else None, P(s_ref), P(l_ref))
    got_s, got_l = host(ds), host(lw)
    # learned: the filter kernels form the hidden activations in packed BF16
    # with the hardware tanh; the oracle rounds the same steps to BF16 with
    # an exact tanh, so activations differ by BF16 units and the network
    # outputs (m, l) by ~1e-3.  That moves a proposal draw nu by up to
    # about 5e-3 (state atol) and the proposal term of the weight,
    # 0.5 (e^2 - nu^2) + 0.5 l summed over four coordinates, by a few 1e-3
    # (median) and a few 1e-2 in the tail.  A wrong move or weight formula
    # moves most particles by 0.1 or more.
    if learned:
        np.testing.assert_allclose(got_s, s_ref, rtol=2e-3, atol=5e-3)
        dl = np.abs(got_l.astype(np.float64) - l_ref)
        assert np.median(dl) < 5e-3, np.median(dl)
        assert np.quantile(dl, 0.99) < 6e-2, np.quantile(dl, 0.99)
        assert dl.max() < 0.3, dl.max()
    else:
        np.testing.assert_allclose(got_s, s_ref, rtol=1e-5, atol=1e-5)
        # the bearing error is small against atan2's value: relative 1e-4
        np.testing.assert_allclose(got_l, l_ref, rtol=1e-4, atol=1e-2)


def _bearings_obs(vc, port, T, seed=0):
    tr = np.zeros(4 * T)
    ob = np.zeros(T)
    port.vo_bearings_simulate(seed, T, ctypes.byref(_omodel()), P(tr), P(ob))
    return ob, tr.reshape(T, 4)


def _oracle_bearings(port, N, T, seed, obs, params=None, prec=32):
    mean = np.zeros(2 * T)
    ess = np.zeros(T)
    res = np.zeros(T, np.int32)
    logz = np.zeros(T)
    port.vo_bearings_pf_run(prec, N, T, seed, 1, 0.5,
                            ctypes.byref(_omodel()), P(obs),
                            P(params) if params is not None else None, 0,
                            P(mean), P(ess), P(res), P(logz))
    return {"mean": mean.reshape(T, 2), "ess": ess, "resampled": res,
            "logz": logz}


@pytest.mark.parametrize("learned", [False, True])
def test_bearings_batch_tracks_oracle(vc, port, learned):
    """Batched bearings filters against the oracle's FP32 filter with the
    same streams.  Step 0 agrees to FP32 rounding.  After it the bearing
    likelihood (sd 0.005 rad) is sharp enough that FP32 differences in the
    normal generator move weights by ~1e-3 relative and change individual
    resampling counts, so the runs are independent Monte Carlo estimates of
    the same posterior: compare them within its spread."""
    T, N = 60, 1 << 13
    obs, truth = _bearings_obs(vc, port, T)
    rng = np.random.default_rng(8)
    p = _params(rng, out_scale=0.02)
    prop = _pack(vc, p) if learned else None
    b = vc.FilterBatch([N, 300], [T, 17], [3, 4], bearings=True,
                       packed=prop.packed.data_ptr() if learned else None)
    g = b.run(np.concatenate([obs, obs[:17]]))[0]
    b.close()
    o = _oracle_bearings(port, N, T, 3, obs, p if learned else None)
    assert abs(g["ess"][0] - o["ess"][0]) / o["ess"][0] < 1e-3
    assert abs(g["logz"][0] - o["logz"][0]) < 1e-3
    assert np.abs(g["mean"] - o["mean"]).mean() < 1.0
    assert abs(g["logz"][-1] - o["logz"][-1]) / T < 0.2
    # bearings-only: range along the line of sight is weakly observed, so
    # check the bearing of the estimated position against the truth's
    tb = np.arctan2(truth[:, 1], truth[:, 0])
    for est in (g, o):
        eb = np.arctan2(est["mean"][:, 1], est["mean"][:, 0])
        assert np.abs(eb - tb).mean() < 0.02


def _samples(m, M, T, rng):
    """(features of x_{t-1} and z_t, nu_t) from M simulated tracks, both in
    the bearing frame of z_t (the inputs and targets the trainer forms)."""
    l11 = np.sqrt(m.q * m.dt ** 3 / 3)
    l21 = m.q * m.dt ** 2 / 2 / l11
    l22 = np.sqrt(m.q * m.dt - l21 ** 2)
    x = np.stack([m.x0 + m.sd_pos0 * rng.normal(size=M),
                  m.y0 + m.sd_pos0 * rng.normal(size=M),
                  m.vx0 + m.sd_vel0 * rng.normal(size=M),
                  m.vy0 + m.sd_vel0 * rng.normal(size=M)])
    feats, nus = [], []
    for _ in range(1, T):
        nu = rng.normal(size=(4, M))
        xn = x.copy()
        xn[0] = x[0] + m.dt * x[2] + l11 * nu[0]
        xn[2] = x[2] + l21 * nu[0] + l22 * nu[1]
        xn[1] = x[1] + m.dt * x[3] + l11 * nu[2]
        xn[3] = x[3] + l21 * nu[2] + l22 * nu[3]
        z = np.arctan2(xn[1], xn[0]) + m.sigma_z * rng.normal(size=M)
        sz, cz = np.sin(z), np.cos(z)
        px, py = x[0] + m.dt * x[2], x[1] + m.dt * x[3]
        r = np.hypot(px, py)
        e = (cz * py - sz * px) / (m.sigma_z * np.maximum(r, 1e-6))
        iv = 1 / (1 + np.hypot(x[2], x[3]))
        feats.append(np.stack([(cz * px + sz * py) / (10 + r),
                               0.125 * e / np.sqrt(1 + e * e / 64),
                               (cz * x[2] + sz * x[3]) * iv,
                               (cz * x[3] - sz * x[2]) * iv, sz, cz], axis=1))
        # the noise pairs (x1, y1), (x2, y2) rotated into the frame:
        # (along, along, across, across)
        nus.append(np.stack([cz * nu[0] + sz * nu[2], cz * nu[1] + sz * nu[3],
                             cz * nu[2] - sz * nu[0], cz * nu[3] - sz * nu[1]],
                            axis=1))
        x = xn
    return (np.concatenate(feats).astype(np.float32),
            np.concatenate(nus).astype(np.float32))


def test_training_lowers_loss_and_log_evidence_spread(vc, port):
    """Train the proposal on simulated trajectories of a model whose bearing
    is informative about the one-step noise (dt 1, q 1: one-step position sd
    0.58 against a lateral bearing resolution of ~0.07 near the start).  The
    held-out loss falls, and the learned filter's log-evidence estimate
    varies less over seeds than the bootstrap's at the same particle
    count."""
    m = vc.bearings_model()
    m.dt, m.q, m.sd_vel0 = 1.0, 1.0, 0.5
    om = _omodel()
    om.dt, om.q, om.sd_vel0 = 1.0, 1.0, 0.5
    T = 30
    feat, nu = _samples(m, 2048, 8, np.random.default_rng(9))
    df, dn = dev(feat), dev(nu)
    prop = vc.Proposal(seed=1)
    before = prop.loss(df.data_ptr(), dn.data_ptr(), len(feat))
    prop.train(m, seed=11, ntraj=1 << 15, T=T, batch=1 << 12, steps=600,
               lr=3e-3)
    after = prop.loss(df.data_ptr(), dn.data_ptr(), len(feat))
    assert after < before - 0.3, (before, after)
    N, R = 256, 64
    tr = np.zeros(4 * T)
    ob = np.zeros(T)
    port.vo_bearings_simulate(5, T, ctypes.byref(om), P(tr), P(ob))
    obs_all = np.tile(ob, R)
    sds = {}
    for name, packed in (("bootstrap", None),
                         ("learned", prop.packed.data_ptr())):
        b = vc.FilterBatch([N] * R, [T] * R, np.arange(R) + 100,
                           models=[m] * R, bearings=True, packed=packed)
        out = b.run(obs_all)
        b.close()
        sds[name] = float(np.std([o["logz"][-1] for o in out]))
    assert sds["learned"] < 0.8 * sds["bootstrap"], sds


def _informative_model(vc, sigma_z=None):
    m = vc.bearings_model()
    m.dt, m.q, m.sd_vel0 = 1.0, 1.0, 0.5
    if sigma_z is not None:
        m.sigma_z = sigma_z
    return m


def test_cloud_rows_flat_likelihood_and_determinism(vc):
    """With a bearing that says nothing (sigma_z = 50 rad) every candidate
    weighs the same, so the chosen noise is N(0, I) in the bearing frame;
    the rows are a function of the seed; every input is bounded."""
    m = _informative_model(vc, sigma_z=50.0)
    feat, nu = vc.cloud_rows(m, 3, 8, 64, 12, 8)
    feat2, nu2 = vc.cloud_rows(m, 3, 8, 64, 12, 8)
    assert feat.shape == (8 * 64 * 11, 6) and nu.shape == (8 * 64 * 11, 4)
    assert bool((feat == feat2).all()) and bool((nu == nu2).all())
    f, n = host(feat), host(nu)
    assert np.isfinite(f).all() and np.isfinite(n).all()
    assert np.abs(f[:, :4]).max() <= 1.0
    np.testing.assert_allclose(f[:, 4] ** 2 + f[:, 5] ** 2, 1.0, atol=1e-5)
    se = 1 / np.sqrt(len(n))
    assert np.abs(n.mean(axis=0)).max() < 5 * se, n.mean(axis=0)
    assert np.abs(n.var(axis=0) - 1).max() < 5 * np.sqrt(2) * se, n.var(0)


def test_cloud_rows_pick_noise_toward_the_bearing(vc):
    """With an informative bearing the chosen across-bearing position noise
    pulls the predicted position back toward the observed bearing: it is
    anti-correlated with the predicted lateral offset (input 1), and the
    along-bearing noise is not."""
    m = _informative_model(vc)
    feat, nu = vc.cloud_rows(m, 5, 64, 256, 60, 64)
    f, n = host(feat), host(nu)
    eb = 8 * f[:, 1]
    e = eb / np.sqrt(np.maximum(1 - eb * eb / 64, 1e-6))
    sel = np.abs(e) < 6
    assert np.corrcoef(n[sel, 2], e[sel])[0, 1] < -0.3
    assert abs(np.corrcoef(n[sel, 0], e[sel])[0, 1]) < 0.05


def test_cloud_rows_teach_the_filter_inputs(vc):
    """Trained on simulated trajectories alone, the network meets the
    filter's own inputs (particles off the observed bearing) rarely; with
    the particle-cloud rows added its loss on held-out cloud rows (other
    tracks, other seed) is clearly lower."""
    import torch
    m = _informative_model(vc)
    T = 40
    rows = vc.cloud_rows(m, 12, 256, 128, T, 128)
    hf, hn = vc.cloud_rows(m, 77, 32, 128, T, 128)
    idx = torch.arange(0, hf.shape[0], 7, device="cuda")
    hf, hn = hf[idx].contiguous(), hn[idx].contiguous()
    out = {}
    for name, extra in (("trajectories", None), ("with clouds", rows)):
        prop = vc.Proposal(seed=1)
        prop.train(m, seed=11, ntraj=1 << 15, T=T, batch=1 << 12, steps=800,
                   lr=3e-3, rows=extra)
        out[name] = prop.loss(hf.data_ptr(), hn.data_ptr(), hf.shape[0])
    assert out["with clouds"] < out["trajectories"] - 0.1, out
