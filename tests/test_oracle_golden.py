"""The oracle's C restatement against golden fixtures made by the reference
itself (tests/golden/make_golden.py).  CPU only."""
import ctypes
import os

import numpy as np
import pytest

from conftest import GOLDEN, P


def load(name):
    return np.load(os.path.join(GOLDEN, f"{name}.npz"))


MODEL = None


def _model():
    from oracle.binding import default_model
    return default_model()


def test_rng_words(port):
    g = load("rng_words")
    n = g["philox_bulk0"].shape[-1]
    for b in (0, 1):
        for i, k in enumerate(g["keys32"]):
            for j, c in enumerate(g["ctrs32"]):
                out = np.zeros(n, np.uint32)
                port.vo_philox4x32_words(P(np.ascontiguousarray(k)),
                                         P(np.ascontiguousarray(c)), n, P(out),
                                         b)
                assert np.array_equal(out, g[f"philox_bulk{b}"][i, j])
        for i, k in enumerate(g["keys64"]):
            for j, c in enumerate(g["ctrs64"]):
                out = np.zeros(n, np.uint64)
                port.vo_threefry4x64_words(P(np.ascontiguousarray(k)),
                                           P(np.ascontiguousarray(c)), n,
                                           P(out), b)
                assert np.array_equal(out, g[f"threefry_bulk{b}"][i, j])


def test_philox_known_answer_and_bulk_quirk():
    g = load("rng_words")
    # key 0, counter all ones: the pre-increment wraps to 0 -> Random123 KAT
    w = g["philox_bulk0"][0, 3][:4]
    assert [int(v) for v in w] == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C,
                                   0x9B00DBD8]
    # the bulk path differs from the scalar stream once the low limb wraps
    # inside a generator call (counter 2^32 - 301 start)
    a, b = g["philox_bulk0"][1, 1], g["philox_bulk1"][1, 1]
    assert not np.array_equal(a, b)
    first = int(np.nonzero(a != b)[0][0])
    assert first == 4 * 299  # block whose low limb is all ones


def test_u01(port):
    g = load("u01")
    u32, u64 = g["u32"], g["u64"]
    for lr in range(4):
        a = np.zeros(len(u32))
        port.vo_u01_u32_f64_n(lr, len(u32), P(u32), P(a))
        assert np.array_equal(a, g[f"u32_f64_{lr}"])
        f = np.zeros(len(u32), np.float32)
        port.vo_u01_u32_f32_n(lr, len(u32), P(u32), P(f))
        assert np.array_equal(f, g[f"u32_f32_{lr}"])
        a = np.zeros(len(u64))
        port.vo_u01_u64_f64_n(lr, len(u64), P(u64), P(a))
        assert np.array_equal(a, g[f"u64_f64_{lr}"])


def test_distributions(port):
    g = load("dist")
    key, ctr = g["key"], g["ctr"]
    for eng in (0, 1):
        for batch in (0, 1):
            for n in (7, 1025, 3001):
                a = np.zeros(n)
                port.vo_u01_dist_f64(eng, P(key), P(ctr), n, P(a), batch)
                assert np.array_equal(a, g[f"u01_e{eng}_b{batch}_n{n}"])
                port.vo_normal_f64(eng, P(key), P(ctr), n, 1.5, 2.0, P(a),
                                   batch)
                assert np.array_equal(a, g[f"normal_e{eng}_b{batch}_n{n}"])
                f = np.zeros(n, np.float32)
                port.vo_normal_f32(eng, P(key), P(ctr), n, 1.5, 2.0, P(f),
                                   batch)
                assert np.array_equal(f, g[f"normalf_e{eng}_b{batch}_n{n}"])
        for df in (0.2, 1.0, 1.5, 2.0, 3.0, 10.0, 30.0):
            a = np.zeros(500)
            port.vo_student_t_f64(eng, P(key), P(ctr), 500, df, P(a))
            assert np.array_equal(a, g[f"student_t_e{eng}_df{df}"])
            if df not in (0.2, 1.5, 2.0, 3.0, 10.0):
                continue
            for n in (1, 7, 1025, 2049):
                b = np.zeros(n)
                port.vo_student_t_batch_f64(eng, P(key), P(ctr), 0, n, df,
                                            P(b), None, None)
                assert np.array_equal(
                    b, g[f"student_t_batch_e{eng}_df{df}_n{n}"]), (eng, df, n)


def test_sequences(port):
    g = load("sequences")
    for kind in range(3):
        for N in (1, 2, 5, 1000):
            a = np.zeros(N)
            nxt = np.zeros(4, np.uint32)
            port.vo_u01_sequence(kind, N, P(g["key"]), P(g["ctr"]), P(a),
                                 P(nxt))
            assert np.array_equal(a, g[f"seq{kind}_n{N}"])
            assert np.array_equal(nxt, g[f"seq{kind}_n{N}_next"])


def test_resampling(port):
    g = load("resample")
    for si in range(int(g["nsizes"][0])):
        M, N = (int(v) for v in g[f"mn{si}"])
        w, u = g[f"w{si}"], g[f"u{si}"]
        rep = np.zeros(M, np.int32)
        port.vo_resample_trans_u01_rep(M, N, P(w), P(u), P(rep))
        assert np.array_equal(rep, g[f"u01rep{si}"])
        for scheme in range(6):
            rep = np.zeros(M, np.int32)
            nxt = np.zeros(4, np.uint32)
            port.vo_resample_words(scheme, M, N, P(g["key"]), P(g["ctr"]),
                                   P(w), P(rep), P(nxt))
            assert np.array_equal(rep, g[f"scheme{scheme}_{si}"])
            assert np.array_equal(nxt, g[f"scheme{scheme}_{si}_next"])
            key = f"scheme{scheme}_{si}_idx"
            if key in g:
                idx = np.zeros(N, np.int32)
                port.vo_resample_trans_rep_index(M, N, P(rep), P(idx))
                assert np.array_equal(idx, g[key])
        resid = np.zeros(M)
        integ = np.zeros(M, np.int32)
        R = port.vo_resample_trans_residual(M, max(N, 1), P(w), P(resid),
                                            P(integ))
        assert R == int(g[f"residR{si}"][0])
        assert np.array_equal(integ, g[f"integ{si}"])
        assert np.array_equal(resid, g[f"resid{si}"], equal_nan=True)


def test_weights(port):
    g = load("weight")
    for n in (1, 3, 1025, 5000):
        W = np.zeros(n)
        ess = port.vo_weight_set_log(n, P(g[f"lw{n}"]), P(W))
        assert np.array_equal(W, g[f"W{n}"]) and ess == g[f"ess{n}"][0]
        W2 = np.zeros(n)
        ess = port.vo_weight_add_log(n, P(W), P(g[f"l{n}"]), P(W2))
        assert np.array_equal(W2, g[f"W2_{n}"]) and ess == g[f"ess2_{n}"][0]
        W3 = np.zeros(n)
        ess = port.vo_weight_set(n, P(g[f"w{n}"]), P(W3))
        assert np.array_equal(W3, g[f"W3_{n}"]) and ess == g[f"ess3_{n}"][0]


def test_filter_runs(port):
    g = load("pf")
    T = g["obs"].shape[0]
    truth = np.zeros(4 * T)
    obs = np.zeros(2 * T)
    port.vo_pf_simulate(0, T, ctypes.byref(_model()), P(truth), P(obs))
    assert np.array_equal(obs.reshape(T, 2), g["obs"])
    assert np.array_equal(truth.reshape(T, 4), g["truth"])
    for prec in (64, 32):
        for scheme in (1, 2):
            n, TT = 4096, 50
            mean = np.zeros(2 * TT)
            ess = np.zeros(TT)
            res = np.zeros(TT, np.int32)
            logz = np.zeros(TT)
            port.vo_pf_run(prec, n, TT, 3, scheme, 0.5,
                           ctypes.byref(_model()), P(obs), 0, P(mean), P(ess),
                           P(res), P(logz))
            tag = f"p{prec}_s{scheme}"
            assert np.array_equal(mean.reshape(TT, 2), g[f"{tag}_mean"])
            assert np.array_equal(ess, g[f"{tag}_ess"])
            assert np.array_equal(res, g[f"{tag}_res"])
            assert np.array_equal(logz, g[f"{tag}_logz"])


def test_oracle_vs_reference_native_streams_statistically(port):
    """The (key = step, counter = particle) streams of the port against the
    reference's own per-particle engines, config 1 (N = 2^14, T = 100,
    stratified, FP64): the log-evidence over 8 port seeds must sit within
    the 64-seed spread of the reference."""
    g = load("pf")
    obs = np.ascontiguousarray(g["obs"])
    T = obs.shape[0]
    ref = g["native64_logz"]
    mu, sd = ref.mean(), ref.std(ddof=1)
    vals = []
    for seed in range(8):
        mean = np.zeros(2 * T)
        ess = np.zeros(T)
        res = np.zeros(T, np.int32)
        logz = np.zeros(T)
        port.vo_pf_run(64, 1 << 14, T, seed, 1, 0.5, ctypes.byref(_model()),
                       P(obs), 0, P(mean), P(ess), P(res), P(logz))
        vals.append(logz[-1])
    vals = np.array(vals)
    # mean of 8 within 4 standard errors; every run within 5 sd
    assert abs(vals.mean() - mu) < 4 * sd / np.sqrt(8) + 4 * sd / np.sqrt(64)
    assert np.all(np.abs(vals - mu) < 5 * sd)


@pytest.mark.skipif(not os.path.exists(os.path.join(
    os.path.dirname(GOLDEN), "..", "oracle", "_ref", "libvsmcref.so")),
    reason="reference build not present on this host")
def test_port_vs_reference_random(port):
    """Random inputs through both the port and the reference build."""
    from oracle import binding
    R = binding.ref()
    rng = np.random.default_rng(99)
    for _ in range(5):
        M = int(rng.integers(2, 5000))
        N = int(rng.integers(1, 5000))
        w = np.exp(rng.normal(0, 3, M))
        w /= w.sum()
        k2 = rng.integers(0, 2**32, 2, dtype=np.uint64).astype(np.uint32)
        c4 = rng.integers(0, 2**32, 4, dtype=np.uint64).astype(np.uint32)
        for scheme in range(6):
            a = np.zeros(M, np.int32)
            b = np.zeros(M, np.int32)
            na = np.zeros(4, np.uint32)
            nb = np.zeros(4, np.uint32)
            R.ref_resample(scheme, M, N, P(k2), P(c4), P(w), P(a), P(na))
            port.vo_resample_words(scheme, M, N, P(k2), P(c4), P(w), P(b),
                                   P(nb))
            assert np.array_equal(a, b) and np.array_equal(na, nb)


def test_numpy_philox_restatement_matches_oracle(port):
    """The tests' vectorized Philox4x32-10 (conftest.philox4x32_10, used for
    float64 restatements of the FP32 kernels) against the oracle's engine:
    word k of an engine at counter {0, i, 0, 0} is block {1 + k // 4, i}."""
    from conftest import P, philox4x32_10
    key = np.array([7, 99], np.uint32)
    for i in (0, 12345, 0xFFFFFFFF):
        ctr = np.array([0, i, 0, 0], np.uint32)
        want = np.zeros(8, np.uint32)
        port.vo_philox4x32_words(P(key), P(ctr), 8, P(want), 0)
        got = []
        for b in (1, 2):
            got += [int(g[0]) for g in philox4x32_10([[b], [i], [0], [0]],
                                                     7, 99)]
        assert got == [int(w) for w in want]
