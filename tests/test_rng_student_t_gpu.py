"""vsmc_cuda_rng_student_t: the engine-advancing batch Student-t of the
reference's C ABI (vsmc_rng_student_t -> student_t_distribution,
rng/student_t_distribution.hpp:97-128), against the oracle's restatement
(itself pinned to the reference's outputs in tests/golden/dist.npz) and
against those fixtures directly.

Every gamma algorithm of the reference is covered: T (df 0.2, alpha < 0.6),
W (df 1.5), E (df 2) and N (df 3, 10); both engines; chunk boundaries
(n = 1, 7, 1025, 2049, 5000); an engine that has already handed out 1 to 3
words of its buffered block; a counter whose low limb wraps inside a bulk
call.  Values agree to 1e-12 relative (CUDA's log / exp / sqrt / sincos
against the host libm), and the engine state after the call is exactly the
oracle's."""
import ctypes

import numpy as np
import pytest

from conftest import GOLDEN, P

pytestmark = pytest.mark.gpu

DFS = (0.2, 1.5, 2.0, 3.0, 10.0)


def _gpu(vc, kind, key, ctr, skip, n, df):
    import torch
    r = vc.rng(kind, key=list(key), ctr=list(ctr))
    if skip:
        buf = torch.zeros(8, dtype=torch.int64, device="cuda")
        vc.call("vsmc_cuda_rng_rand", ctypes.byref(r), skip, buf.data_ptr(),
                None)
    out = torch.zeros(max(n, 1), dtype=torch.float64, device="cuda")
    vc.call("vsmc_cuda_rng_student_t", ctypes.byref(r), n, out.data_ptr(),
            ctypes.c_double(df), None)
    torch.cuda.synchronize()
    return out.cpu().numpy()[:n], [int(c) for c in r.ctr], int(r.index)


def _oracle(port, eng, key, ctr, skip, n, df):
    k = np.array(list(key) + [0] * (4 - len(key)), np.uint64)
    c = np.array(list(ctr) + [0] * (4 - len(ctr)), np.uint64)
    out = np.zeros(max(n, 1))
    co = np.zeros(4, np.uint64)
    idx = np.zeros(1, np.uint32)
    port.vo_student_t_batch_f64(eng, P(k), P(c), skip, n, df, P(out), P(co),
                                P(idx))
    return out[:n], [int(v) for v in co], int(idx[0])


def _close(a, b):
    return np.allclose(a, b, rtol=1e-12, atol=1e-300) and \
        np.array_equal(np.isnan(a), np.isnan(b))


@pytest.mark.parametrize("df", DFS)
@pytest.mark.parametrize("eng", [0, 1])
def test_student_t_engine_matches_oracle(vc, port, eng, df):
    kind = vc.PHILOX4X32 if eng == 0 else vc.THREEFRY4X64
    key = (5, 7) if eng == 0 else (5, 7, 11, 13)
    for n in (1, 7, 1025, 2049, 5000):
        for skip in (0, 1, 3):
            ctr = (3, 1, 0, 0)
            g, gc, gi = _gpu(vc, kind, key, ctr, skip, n, df)
            o, oc, oi = _oracle(port, eng, key, ctr, skip, n, df)
            assert _close(g, o), (n, skip, np.abs(g - o).max())
            # the engine advanced by the reference's words
            assert gc == oc and gi == oi, (n, skip, gc, oc, gi, oi)


@pytest.mark.parametrize("df", DFS)
@pytest.mark.parametrize("eng", [0, 1])
def test_student_t_engine_matches_reference_fixtures(vc, eng, df):
    g = np.load(f"{GOLDEN}/dist.npz")
    kind = vc.PHILOX4X32 if eng == 0 else vc.THREEFRY4X64
    key = [int(v) for v in g["key"]]
    ctr = [int(v) for v in g["ctr"]]
    if eng == 0:
        key = key[:2]
    for n in (1, 7, 1025, 2049):
        want = g[f"student_t_batch_e{eng}_df{df}_n{n}"]
        got, _, _ = _gpu(vc, kind, key, ctr, 0, n, df)
        assert _close(got, want), (n, np.abs(got - want).max())


def test_student_t_engine_counter_wrap(vc, port):
    """The low counter limb passes all ones inside the bulk calls (the
    reference's extra limb-1 carry at an all-ones low limb)."""
    for eng, kind, key, ctr in (
            (0, vc.PHILOX4X32, (9, 4), (0xFFFFFFFF - 300, 2, 0, 0)),
            (1, vc.THREEFRY4X64, (9, 4, 1, 2), (2**64 - 300, 7, 0, 0))):
        for df in (1.5, 10.0):
            g, gc, gi = _gpu(vc, kind, key, ctr, 2, 3001, df)
            o, oc, oi = _oracle(port, eng, key, ctr, 2, 3001, df)
            assert _close(g, o)
            assert gc == oc and gi == oi


def test_student_t_engine_long_run(vc, port):
    """2^17 variates (128 chunks in sequence), df = 3 (algorithm N, whose
    v <= 0 redraws occur at this alpha)."""
    n = 1 << 17
    g, gc, gi = _gpu(vc, vc.PHILOX4X32, (1, 2), (0, 0, 0, 0), 0, n, 3.0)
    o, oc, oi = _oracle(port, 0, (1, 2), (0, 0, 0, 0), 0, n, 3.0)
    assert _close(g, o), np.abs(g - o).max()
    assert gc == oc and gi == oi


def test_student_t_engine_rejects_bad_arguments(vc):
    L = vc.lib()
    r = vc.rng(vc.PHILOX4X32, seed=1)
    import torch
    out = torch.zeros(4, dtype=torch.float64, device="cuda")
    assert L.vsmc_cuda_rng_student_t(ctypes.byref(r), 4, out.data_ptr(),
                                     0.0, None) == vc.ERR_ARG
    assert L.vsmc_cuda_rng_student_t(None, 4, out.data_ptr(), 3.0,
                                     None) == vc.ERR_ARG
    assert L.vsmc_cuda_rng_student_t(ctypes.byref(r), 0, None, 3.0,
                                     None) == 0
