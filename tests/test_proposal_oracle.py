"""The proposal network's oracle (CPU): its backpropagation against central
finite differences of its own loss in exact FP64, and the BF16 rounding mode
staying close to exact."""
import ctypes

import numpy as np

from conftest import P


def _params(rng, scale=0.3):
    npar = 64 * 6 + 64 + 64 * 64 + 64 + 8 * 64 + 8
    return (rng.normal(0, scale, npar)).astype(np.float32)


def _data(rng, B):
    feat = rng.normal(0, 1, (B, 6)).astype(np.float32)
    nu = rng.normal(0, 1, (B, 4)).astype(np.float32)
    return feat, nu


def test_oracle_gradient_matches_finite_differences(port):
    rng = np.random.default_rng(3)
    p = _params(rng)
    feat, nu = _data(rng, 7)
    port.vo_mlp_set_rounding(0)
    try:
        loss = ctypes.c_double()
        grad = np.zeros(p.size)
        port.vo_mlp_loss_grad(P(p), 7, P(feat), P(nu), ctypes.byref(loss),
                              P(grad))
        idx = rng.choice(p.size, 60, replace=False)
        idx = np.concatenate([idx, [0, 383, 384, 447, 448, 4543, 4544,
                                    4607, 4608, 5119, 5120, 5127]])
        for i in idx:
            h = 1e-3 * max(1.0, abs(float(p[i])))
            lp, lm = ctypes.c_double(), ctypes.c_double()
            g = np.zeros(p.size)
            q = p.astype(np.float64)
            for sign, out in ((1, lp), (-1, lm)):
                pp = q.copy()
                pp[i] += sign * h
                pf = pp.astype(np.float32)
                port.vo_mlp_loss_grad(P(pf), 7, P(feat), P(nu),
                                      ctypes.byref(out), P(g))
            # the parameter itself is rounded to float: use the realised step
            hp = float(np.float32(q[i] + h)) - float(q[i])
            hm = float(q[i]) - float(np.float32(q[i] - h))
            fd = (lp.value - lm.value) / (hp + hm)
            assert abs(fd - grad[i]) <= 2e-4 * max(1.0, abs(grad[i])), (
                i, fd, grad[i])
    finally:
        port.vo_mlp_set_rounding(1)


def test_device_rounding_stays_near_exact(port):
    rng = np.random.default_rng(4)
    p = _params(rng)
    feat, nu = _data(rng, 64)
    out_r = np.zeros((64, 8), np.float32)
    port.vo_mlp_forward(P(p), 64, P(feat), P(out_r))
    port.vo_mlp_set_rounding(0)
    try:
        out_e = np.zeros((64, 8), np.float32)
        port.vo_mlp_forward(P(p), 64, P(feat), P(out_e))
    finally:
        port.vo_mlp_set_rounding(1)
    # BF16 operands (8-bit mantissa) on a 64-wide sum: a few 1e-3 relative
    err = np.abs(out_r - out_e) / (1 + np.abs(out_e))
    assert err.max() < 3e-2
    assert err.mean() < 5e-3
