"""Resampling at the microbenchmark size: N = 2^24 weights with log w iid
N(0, 3^2), normalized in FP64, all six schemes through the C ABI
(vsmc_cuda_resample) against the oracle (pinned to the reference), for the
same weights and the same engine.

* Stratified, systematic, residual-stratified and residual-systematic:
  replication counts bit-exact, engine advanced by exactly the reference's
  words.
* Multinomial and residual draw sorted uniforms (rng/u01_sequence.hpp:
  131-164) whose log / exp come from CUDA's libm on the device and from the
  host's libm in the reference, so a uniform can differ in its last bits.
  Every count mismatch must be explained by such a uniform falling on the
  other side of a CDF boundary: the test rebuilds both runs' parent of every
  uniform with the reference's two-pointer rule (resample/transform.hpp:
  43-71), checks that they reproduce both count vectors exactly, and reports
  the uniforms that cross, with their distance to the boundary in ulps."""
import ctypes

import numpy as np
import pytest

from conftest import P, dev, host

pytestmark = pytest.mark.gpu

N = 1 << 24
EXACT = {1, 2, 4, 5}
NAMES = ["multinomial", "stratified", "systematic", "residual",
         "residual_stratified", "residual_systematic"]


@pytest.fixture(scope="module")
def weights():
    rng = np.random.default_rng(20240)
    lw = rng.normal(0, 3.0, N)
    w = np.exp(lw - lw.max())
    return w / w.sum()


def _parents(cdf, u):
    """Parent of each sorted uniform under the two-pointer rule: the first
    i < M - 1 with u <= cdf_i, else M - 1."""
    return np.searchsorted(cdf[:-1], u, side="left")


def _ulps(a, b):
    return np.abs(a - b) / np.spacing(np.maximum(np.abs(a), np.abs(b)))


@pytest.mark.parametrize("scheme", range(6))
def test_schemes_at_2_to_24(vc, port, weights, scheme):
    import torch
    w = weights
    key = np.array([2024, 7], np.uint32)
    ctr = np.array([0xFFFFFF00, 0, 0, 0], np.uint32)
    rep_ref = np.zeros(N, np.int32)
    next_ref = np.zeros(4, np.uint32)
    port.vo_resample_words(scheme, N, N, P(key), P(ctr), P(w), P(rep_ref),
                           P(next_ref))
    r = vc.rng(vc.PHILOX4X32, key=[2024, 7], ctr=[0xFFFFFF00, 0, 0, 0])
    rep = torch.zeros(N, dtype=torch.int32, device="cuda")
    vc.call("vsmc_cuda_resample", N, N, ctypes.byref(r), dev(w).data_ptr(),
            rep.data_ptr(), scheme, None)
    got = host(rep)
    nxt = torch.zeros(4, dtype=torch.int32, device="cuda")
    vc.call("vsmc_cuda_rng_rand", ctypes.byref(r), 4, nxt.data_ptr(), None)
    assert np.array_equal(host(nxt).view(np.uint32), next_ref), "engine"
    assert got.sum() == N
    if scheme in EXACT:
        assert np.array_equal(got, rep_ref)
        return

    # the sorted-uniform schemes: rebuild both runs from their uniforms
    if scheme == 0:
        base = np.zeros(N, np.int32)
        cw = w
        R = N
    else:
        resid = np.zeros(N)
        integ = np.zeros(N, np.int32)
        R = port.vo_resample_trans_residual(N, N, P(w), P(resid), P(integ))
        base = integ
        cw = resid
    words = np.zeros(R, np.uint32)
    port.vo_philox4x32_words(P(key), P(ctr), R, P(words), 0)
    u01 = words.astype(np.float64) * 2.0**-32
    u_ref = np.zeros(R)
    port.vo_u01_sorted(R, P(u01), P(u_ref))
    ud = torch.zeros(R, dtype=torch.float64, device="cuda")
    vc.call("vsmc_cuda_u01_sorted", R, dev(u01).data_ptr(), ud.data_ptr(),
            None)
    u_gpu = host(ud)
    cdf = np.cumsum(cw)  # left to right, as the reference sums
    p_ref = _parents(cdf, u_ref)
    p_gpu = _parents(cdf, u_gpu)
    assert np.array_equal(base + np.bincount(p_ref, minlength=N), rep_ref)
    assert np.array_equal(base + np.bincount(p_gpu, minlength=N), got)
    differ = np.flatnonzero(u_gpu != u_ref)
    cross = np.flatnonzero(p_gpu != p_ref)
    mism = np.flatnonzero(got != rep_ref)
    # each crossing uniform straddles the boundary it crosses: the CDF value
    # between its two versions, within their distance of both
    lo = np.minimum(p_gpu[cross], p_ref[cross])
    b = cdf[lo]
    a1, a2 = u_gpu[cross], u_ref[cross]
    assert np.all((np.minimum(a1, a2) <= b) & (b <= np.maximum(a1, a2)))
    dist = _ulps(np.where(np.abs(a1 - b) < np.abs(a2 - b), a1, a2), b) \
        if len(cross) else np.zeros(0)
    # u = 1 - exp(l): the difference of the two libm's exp results near 1,
    # in units of 2^-53 (a few), and so in absolute terms, not in ulps of u
    du = np.abs(u_gpu - u_ref).max() / 2.0**-53
    print(f"{NAMES[scheme]} N=2^24: {len(differ)} of {R} sorted uniforms "
          f"differ (max |du| = {du:.1f} x 2^-53); {len(cross)} cross a CDF "
          f"boundary (within {dist.max() if len(cross) else 0:.0f} ulp of "
          f"it); {len(mism)} counts differ")
    assert du <= 64, du
    assert len(cross) <= 4, len(cross)
