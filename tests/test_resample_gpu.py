"""Exact FP64 resampling path vs the oracle: left-to-right sums, u01 -> rep,
rep -> index, residual split, the six schemes with engine consumption, the
particle copy, the Weight operations and the monitor mean."""
import ctypes

import numpy as np
import pytest

from conftest import P, dev, host

pytestmark = pytest.mark.gpu


def _weights(rng, m, sd=3.0):
    lw = rng.normal(0, sd, m)
    w = np.exp(lw - lw.max())
    return w / w.sum()


def _seqsum_gpu(vc, x):
    import torch
    n = len(x)
    dx = dev(x)
    pre = torch.zeros(max(n, 1), dtype=torch.float64, device="cuda")
    tot = torch.zeros(1, dtype=torch.float64, device="cuda")
    vc.call("vsmc_cuda_sequential_sum", n, dx.data_ptr(), pre.data_ptr(),
            tot.data_ptr(), None)
    return host(pre)[:n], host(tot)[0]


def _seq_cumsum(x):
    # np.cumsum on float64 adds left to right (a sequential loop)
    out = np.empty_like(x)
    s = 0.0
    for i, v in enumerate(x):
        s += v
        out[i] = s
    return out


@pytest.mark.parametrize("case", ["lognormal", "uniform", "zeros", "ties",
                                  "tiny", "huge_range", "one", "two"])
def test_sequential_sum_bit_exact(vc, case):
    rng = np.random.default_rng(7)
    if case == "lognormal":
        x = _weights(rng, 200000)
    elif case == "uniform":
        x = rng.random(100003)
    elif case == "zeros":
        x = rng.random(5000)
        x[rng.random(5000) < 0.5] = 0.0
        x[:100] = 0.0
    elif case == "ties":
        # running sums sitting on odd multiples of the ulp with half-ulp
        # increments: round-half-even decides
        x = np.array([1.0, 2.0**-52] + [2.0**-53] * 50 + [2.0**-52, 2.0**-53]
                     * 50 + [3 * 2.0**-53] * 40)
    elif case == "tiny":
        x = rng.random(3000) * 1e-300
    elif case == "huge_range":
        x = np.exp(rng.normal(0, 30, 20000))
    elif case == "one":
        x = np.array([0.3])
    else:
        x = np.array([0.1, 0.2])
    want = np.cumsum(x) if len(x) > 300 else _seq_cumsum(x)
    got, tot = _seqsum_gpu(vc, x)
    assert np.array_equal(got, want)
    assert tot == want[-1]


def test_sequential_sum_matches_python_loop_exactly(vc):
    rng = np.random.default_rng(3)
    x = _weights(rng, 4000, 5.0)
    got, _ = _seqsum_gpu(vc, x)
    assert np.array_equal(got, _seq_cumsum(x))


def test_sequential_sum_rejects_negative(vc):
    import torch
    x = dev(np.array([0.5, -1.0, 0.2]))
    tot = torch.zeros(1, dtype=torch.float64, device="cuda")
    rc = vc.lib().vsmc_cuda_sequential_sum(3, x.data_ptr(), None,
                                           tot.data_ptr(), None)
    assert rc == vc.ERR_NONFINITE


SIZES = [(1, 5), (5, 0), (2, 3), (3, 1), (100, 100), (1000, 1000),
         (1000, 700), (700, 1000), (50000, 50000)]


@pytest.mark.parametrize("m,n", SIZES)
@pytest.mark.parametrize("kind", ["sorted", "unsorted"])
def test_trans_u01_rep_and_index(vc, port, m, n, kind):
    import torch
    rng = np.random.default_rng(m * 7 + n)
    w = _weights(rng, m)
    u = rng.random(max(n, 1))[:n]
    if kind == "sorted":
        u = np.sort(u)
    rep_ref = np.zeros(m, np.int32)
    port.vo_resample_trans_u01_rep(m, n, P(w), P(u), P(rep_ref))
    rep = torch.zeros(max(m, 1), dtype=torch.int32, device="cuda")
    du = dev(u) if n else None
    vc.call("vsmc_cuda_resample_trans_u01_rep", m, n, dev(w).data_ptr(),
            du.data_ptr() if n else None, rep.data_ptr(), None)
    assert np.array_equal(host(rep)[:m], rep_ref)
    if n and m:
        idx_ref = np.zeros(n, np.int32)
        port.vo_resample_trans_u01_index(m, n, P(w), P(u), P(idx_ref))
        idx = torch.zeros(n, dtype=torch.int32, device="cuda")
        vc.call("vsmc_cuda_resample_trans_u01_index", m, n, dev(w).data_ptr(),
                du.data_ptr(), idx.data_ptr(), None)
        assert np.array_equal(host(idx), idx_ref)


def test_trans_u01_rep_large_exact(vc, port):
    """N = 2^20, log-weights N(0, 3^2): counts identical for identical
    weights and uniforms (the CDF is the reference's left-to-right sum)."""
    import torch
    rng = np.random.default_rng(11)
    m = n = 1 << 20
    w = _weights(rng, m)
    u = (rng.random(n) + np.arange(n)) / n  # stratified-like sorted uniforms
    rep_ref = np.zeros(m, np.int32)
    port.vo_resample_trans_u01_rep(m, n, P(w), P(u), P(rep_ref))
    rep = torch.zeros(m, dtype=torch.int32, device="cuda")
    vc.call("vsmc_cuda_resample_trans_u01_rep", m, n, dev(w).data_ptr(),
            dev(u).data_ptr(), rep.data_ptr(), None)
    got = host(rep)
    assert np.array_equal(got, rep_ref), int((got != rep_ref).sum())


@pytest.mark.parametrize("m,n", [(1, 1), (4, 4), (1000, 1000), (300, 500),
                                 (500, 300), (100000, 100000)])
def test_rep_index_and_back(vc, port, m, n):
    import torch
    rng = np.random.default_rng(m + n)
    if m == n:
        rep = rng.multinomial(n, _weights(rng, m, 2.0)).astype(np.int32)
    else:
        rep = rng.multinomial(min(n, m * 3), np.ones(m) / m).astype(np.int32)
        rep = rep[:m]
    tot = int(rep.sum())
    idx_ref = np.zeros(n, np.int32)
    port.vo_resample_trans_rep_index(m, n, P(rep), P(idx_ref))
    idx = torch.zeros(n, dtype=torch.int32, device="cuda")
    vc.call("vsmc_cuda_resample_trans_rep_index", m, n, dev(rep).data_ptr(),
            idx.data_ptr(), None)
    got = host(idx)
    cnt = n if m == n else tot
    assert np.array_equal(got[:cnt], idx_ref[:cnt])
    if m == n:
        back = torch.zeros(m, dtype=torch.int32, device="cuda")
        vc.call("vsmc_cuda_resample_trans_index_rep", m, n, idx.data_ptr(),
                back.data_ptr(), None)
        ref_back = np.zeros(m, np.int32)
        port.vo_resample_trans_index_rep(m, n, P(idx_ref), P(ref_back))
        assert np.array_equal(host(back), ref_back)
        assert np.array_equal(host(back), rep)


def test_rep_index_rejects_bad_counts(vc):
    import torch
    rep = dev(np.array([2, 2, 0], np.int32))  # sums to 4 != 3
    idx = torch.zeros(3, dtype=torch.int32, device="cuda")
    rc = vc.lib().vsmc_cuda_resample_trans_rep_index(3, 3, rep.data_ptr(),
                                                    idx.data_ptr(), None)
    assert rc == vc.ERR_ARG


@pytest.mark.parametrize("m,n", [(10, 10), (1000, 1000), (1000, 3000),
                                 (65537, 65537)])
def test_residual_split(vc, port, m, n):
    import torch
    rng = np.random.default_rng(m)
    w = _weights(rng, m)
    resid_ref = np.zeros(m)
    integ_ref = np.zeros(m, np.int32)
    R_ref = port.vo_resample_trans_residual(m, n, P(w), P(resid_ref),
                                            P(integ_ref))
    resid = torch.zeros(m, dtype=torch.float64, device="cuda")
    integ = torch.zeros(m, dtype=torch.int32, device="cuda")
    R = ctypes.c_size_t(0)
    vc.call("vsmc_cuda_resample_trans_residual", m, n, dev(w).data_ptr(),
            resid.data_ptr(), integ.data_ptr(), ctypes.byref(R), None)
    assert R.value == R_ref
    assert np.array_equal(host(integ), integ_ref)
    assert np.array_equal(host(resid), resid_ref)


# n a power of two (1, 4096, 2^18) takes the integer path of the
# stratified / systematic uniforms; the others the FP64 one
SCHEME_SIZES = [(1, 5), (5, 0), (2, 3), (64, 1), (100, 100), (1000, 1000),
                (1000, 700), (4096, 4096), (50000, 50000), (1 << 18, 1 << 18)]
EXACT = {1, 2, 4, 5}  # stratified, systematic and their residual forms


@pytest.mark.parametrize("scheme", range(6))
@pytest.mark.parametrize("m,n", SCHEME_SIZES)
def test_schemes_counts_and_engine(vc, port, scheme, m, n):
    import torch
    rng = np.random.default_rng(1000 * scheme + m + n)
    w = _weights(rng, m)
    key = np.array([9, 11], np.uint32)
    ctr = np.array([0xFFFFFFF0, 2, 0, 0], np.uint32)
    rep_ref = np.zeros(m, np.int32)
    next_ref = np.zeros(4, np.uint32)
    port.vo_resample_words(scheme, m, n, P(key), P(ctr), P(w), P(rep_ref),
                           P(next_ref))
    r = vc.rng(vc.PHILOX4X32, key=[9, 11], ctr=[0xFFFFFFF0, 2, 0, 0])
    rep = torch.zeros(m, dtype=torch.int32, device="cuda")
    vc.call("vsmc_cuda_resample", m, n, ctypes.byref(r), dev(w).data_ptr(),
            rep.data_ptr(), scheme, None)
    got = host(rep)
    nxt = torch.zeros(4, dtype=torch.int32, device="cuda")
    vc.call("vsmc_cuda_rng_rand", ctypes.byref(r), 4, nxt.data_ptr(), None)
    assert np.array_equal(host(nxt).view(np.uint32), next_ref), "engine"
    assert got.sum() == n
    if scheme in EXACT:
        assert np.array_equal(got, rep_ref)
    else:
        # sorted uniforms use CUDA's log / exp: a uniform may differ from the
        # reference's in its last bit, which can move one copy across a CDF
        # boundary; such moves must be rare and local
        diff = np.abs(got - rep_ref)
        assert diff.sum() <= 2 * max(1, m // 20000), diff.sum()


def test_u01_sequence_arrays(vc, port):
    import torch
    rng = np.random.default_rng(5)
    for n in (1, 2, 1000, 100001):
        u = rng.random(n)
        for name, fn in (("stratified", port.vo_u01_stratified),
                         ("sorted", port.vo_u01_sorted)):
            ref = np.zeros(n)
            fn(n, P(u), P(ref))
            out = torch.zeros(n, dtype=torch.float64, device="cuda")
            vc.call(f"vsmc_cuda_u01_{name}", n, dev(u).data_ptr(),
                    out.data_ptr(), None)
            got = host(out)
            if name == "stratified":
                assert np.array_equal(got, ref)
            else:
                np.testing.assert_allclose(got, ref, rtol=1e-13, atol=1e-15)
        ref = np.zeros(n)
        port.vo_u01_systematic(n, float(u[0]), P(ref))
        out = torch.zeros(n, dtype=torch.float64, device="cuda")
        vc.call("vsmc_cuda_u01_systematic", n, float(u[0]), out.data_ptr(),
                None)
        assert np.array_equal(host(out), ref)


@pytest.mark.parametrize("prec", [32, 64])
def test_state_copy_in_place(vc, port, prec):
    import torch
    rng = np.random.default_rng(prec)
    n = 20000
    rep = rng.multinomial(n, _weights(rng, n, 2.0)).astype(np.int32)
    idx = np.zeros(n, np.int32)
    port.vo_resample_trans_rep_index(n, n, P(rep), P(idx))
    dt = np.float32 if prec == 32 else np.float64
    state = rng.normal(0, 1, (4, n)).astype(dt)
    ref = state.copy()
    (port.vo_state_copy_f32 if prec == 32 else port.vo_state_copy_f64)(
        n, P(idx), P(ref))
    ds = dev(state)
    vc.call(f"vsmc_cuda_state_copy_f{prec}", n, 4, dev(idx).data_ptr(),
            ds.data_ptr(), None)
    assert np.array_equal(host(ds), ref)
    # an index array that moves a source slot is rejected
    bad = dev(np.array([1, 0, 2], np.int32))
    rc = getattr(vc.lib(), f"vsmc_cuda_state_copy_f{prec}")(
        3, 4, bad.data_ptr(), ds.data_ptr(), None)
    assert rc == vc.ERR_ARG


@pytest.mark.parametrize("n", [1, 3, 1024, 1025, 100000])
def test_weights(vc, port, n):
    import torch
    rng = np.random.default_rng(n)
    w = rng.random(n) + 0.01
    ref = np.zeros(n)
    ess_ref = port.vo_weight_set(n, P(w), P(ref))
    W = torch.zeros(n, dtype=torch.float64, device="cuda")
    ess = torch.zeros(1, dtype=torch.float64, device="cuda")
    vc.call("vsmc_cuda_weight_set", n, dev(w).data_ptr(), W.data_ptr(),
            ess.data_ptr(), None)
    assert np.array_equal(host(W), ref)
    assert host(ess)[0] == ess_ref
    # set_log / add_log: CUDA exp / log, 1e-12 relative
    lw = rng.normal(0, 3, n)
    ess_ref = port.vo_weight_set_log(n, P(lw), P(ref))
    vc.call("vsmc_cuda_weight_set_log", n, dev(lw).data_ptr(), W.data_ptr(),
            ess.data_ptr(), None)
    np.testing.assert_allclose(host(W), ref, rtol=1e-12, atol=1e-300)
    assert abs(host(ess)[0] - ess_ref) <= 1e-12 * ess_ref
    l = rng.normal(0, 1, n)
    ref2 = np.zeros(n)
    ess_ref = port.vo_weight_add_log(n, P(ref), P(l), P(ref2))
    vc.call("vsmc_cuda_weight_add_log", n, dev(l).data_ptr(), W.data_ptr(),
            ess.data_ptr(), None)
    np.testing.assert_allclose(host(W), ref2, rtol=1e-11, atol=1e-300)
    assert abs(host(ess)[0] - ess_ref) <= 1e-11 * ess_ref
    # set_equal is exact: normalize(false) of fill(1/N)
    eq = np.full(n, 1.0 / n)
    ess_ref = port.vo_weight_set(n, P(eq), P(ref))
    vc.call("vsmc_cuda_weight_set_equal", n, W.data_ptr(), ess.data_ptr(),
            None)
    assert np.array_equal(host(W), ref)
    assert host(ess)[0] == ess_ref


def test_monitor_mean(vc):
    import torch
    rng = np.random.default_rng(2)
    n = 77777
    W = rng.random(n)
    W /= W.sum()
    s = rng.normal(0, 3, (4, n))
    out = torch.zeros(4, dtype=torch.float64, device="cuda")
    vc.call("vsmc_cuda_monitor_mean_f64", n, 4, dev(s).data_ptr(),
            dev(W).data_ptr(), out.data_ptr(), None)
    np.testing.assert_allclose(host(out), s @ W, rtol=1e-12, atol=1e-12)
    vc.call("vsmc_cuda_monitor_mean_f32", n, 2,
            dev(s.astype(np.float32)).data_ptr(), dev(W).data_ptr(),
            out.data_ptr(), None)
    np.testing.assert_allclose(host(out)[:2], s.astype(np.float32)[:2] @ W,
                               rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("scheme", range(6))
@pytest.mark.parametrize("bad", ["nan", "negative"])
def test_schemes_reject_invalid_weights(vc, scheme, bad):
    """A NaN or negative weight is reported (VSMC_CUDA_ERR_NONFINITE) by
    every scheme, and the host engine is left where it was; the reference
    leaves such input undefined (internal/assert.hpp:42-62)."""
    import torch
    m = n = 1000
    w = np.full(m, 1.0 / m)
    w[417] = np.nan if bad == "nan" else -1.0 / m
    r = vc.rng(vc.PHILOX4X32, key=[3, 4], ctr=[5, 0, 0, 0])
    before = [int(v) for v in r.ctr], r.index
    rep = torch.zeros(m, dtype=torch.int32, device="cuda")
    rc = vc.lib().vsmc_cuda_resample(m, n, ctypes.byref(r), dev(w).data_ptr(),
                                     rep.data_ptr(), scheme, None)
    assert rc == vc.ERR_NONFINITE
    assert ([int(v) for v in r.ctr], r.index) == before


@pytest.mark.parametrize("case", ["wraps_to_zero", "wraps_into_range"])
def test_residual_split_rejects_integer_parts_past_2_to_31(vc, case):
    """Unnormalized weights whose integer parts n * w_i add up past 2^31:
    the total is formed in 64 bits, so a 32-bit wrap back into [0, n]
    cannot pass as a valid draw; the split reports VSMC_CUDA_ERR_ARG."""
    import torch
    n = 4
    if case == "wraps_to_zero":
        w = np.full(4, 2.0**28)          # 4 * 2^30 = 2^32 = 0 mod 2^32
    else:
        w = np.array([2.0**28] * 4 + [0.5])  # 2^32 + 2 = 2 mod 2^32
    m = len(w)
    resid = torch.zeros(m, dtype=torch.float64, device="cuda")
    integ = torch.zeros(m, dtype=torch.int32, device="cuda")
    R = ctypes.c_size_t(0)
    rc = vc.lib().vsmc_cuda_resample_trans_residual(
        m, n, dev(w).data_ptr(), resid.data_ptr(), integ.data_ptr(),
        ctypes.byref(R), None)
    assert rc == vc.ERR_ARG
