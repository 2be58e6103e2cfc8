"""The integer-CDF resampler of the precision-32 filter, bit-exact against a
Python big-integer restatement of its definition: uniform j is
u_j = (j + a_j 2^-32) / n and counts toward the first i with
u_j <= (q_0 + ... + q_i) / Q; the last slot takes the rest; parents keep
their slot and empty slots take surplus copies in order."""
import ctypes

import numpy as np
import pytest

from conftest import P, dev, host

pytestmark = pytest.mark.gpu

KEY = (123, 456)
CTR = (0xFFFFFFF0, 7, 0, 0)


def engine_words(port, k):
    out = np.zeros(k + 4, np.uint32)
    port.vo_philox4x32_words(P(np.array(KEY, np.uint32)),
                             P(np.array(CTR, np.uint32)), len(out), P(out), 0)
    return [int(v) for v in out]


def reference_counts(q, scheme, words):
    n = len(q)
    Q = sum(q)
    two32 = 1 << 32

    def F(c):
        if scheme == 2:  # systematic: one word for all j
            num = c * n * two32 - words[0] * Q
            if num < 0:
                return 0
            return min(n, num // (Q * two32) + 1)
        j0 = min(n, c * n // Q)
        if j0 >= n:
            return n
        r0 = c * n - j0 * Q
        g = -(-(words[j0] * Q) // two32)  # ceil
        return j0 + (1 if g <= r0 else 0)

    rep = []
    prev = 0
    c = 0
    for i in range(n):
        c += q[i]
        f = n if i == n - 1 else F(c)
        rep.append(f - prev)
        prev = f
    return np.array(rep, np.int32)


def brute_counts(q, scheme, words):
    """Direct definition: loop over the uniforms (small n only)."""
    n = len(q)
    Q = sum(q)
    C = np.cumsum(np.array(q, dtype=object))
    rep = np.zeros(n, np.int32)
    i = 0
    for j in range(n):
        a = words[0] if scheme == 2 else words[j]
        while i < n - 1 and (j * 2**32 + a) * Q > int(C[i]) * n * 2**32:
            i += 1
        rep[i] += 1
    return rep


def consumed(rep, scheme):
    if scheme == 2:
        return 1
    n = len(rep)
    jf = n - int(rep[-1])
    return jf + 1 if jf < n else n


@pytest.mark.parametrize("scheme", [1, 2])
@pytest.mark.parametrize("n,kind", [(2, "ln3"), (5, "ln3"), (1000, "ln3"),
                                    (4099, "equal"), (30000, "ln1"),
                                    (30000, "spike"), (250000, "ln3")])
def test_fixed_point_resampler_exact(vc, port, scheme, n, kind):
    import torch
    rng = np.random.default_rng(n + scheme)
    shift = 63 - int(np.ceil(np.log2(n)))
    if kind == "equal":
        w = np.ones(n)
    elif kind == "spike":
        w = np.exp(rng.normal(0, 1, n) - 30)
        w[n // 3] = 1.0
    else:
        lw = rng.normal(0, 3.0 if kind == "ln3" else 1.0, n)
        w = np.exp(lw - lw.max())
    q = np.floor(w * 2.0**shift).astype(np.uint64)
    qi = [int(v) for v in q]
    words = engine_words(port, n)
    ref = reference_counts(qi, scheme, words)
    if n <= 1000:
        assert np.array_equal(ref, brute_counts(qi, scheme, words))
    r = vc.rng(vc.PHILOX4X32, key=list(KEY), ctr=list(CTR))
    rep = torch.zeros(n, dtype=torch.int32, device="cuda")
    idx = torch.zeros(n, dtype=torch.int32, device="cuda")
    dq = dev(q)
    vc.call("vsmc_cuda_resample_fixed", n, dq.data_ptr(), scheme,
            ctypes.byref(r), rep.data_ptr(), idx.data_ptr(), None)
    got = host(rep)
    assert np.array_equal(got, ref), int((got != ref).sum())
    want_idx = np.zeros(n, np.int32)
    port.vo_resample_trans_rep_index(n, n, P(ref), P(want_idx))
    assert np.array_equal(host(idx), want_idx)
    # engine advanced by exactly the words the reference sequence consumes
    k = consumed(ref, scheme)
    total = 4 + k - 1  # engine placed with an exhausted buffer (index 4)
    ctr = list(CTR)
    ctr[0] += total // 4
    carry, ctr[0] = divmod(ctr[0], 2**32)
    ctr[1] += carry
    assert [int(v) for v in r.ctr] == ctr
    assert r.index == total % 4 + 1


def _integer_weights(kind, n, rng):
    """Integer CDFs that put many CDF values on or next to a uniform: small
    totals (every C n / Q a fraction of small denominator), equal and
    power-of-two weights (C n / Q an integer or a fixed fraction), totals
    near 2^63, single weights of 2^62 among tiny ones, and long zero runs."""
    if kind == "tiny":
        return rng.integers(0, 3, n).astype(np.uint64)
    if kind == "equal1":
        return np.ones(n, np.uint64)
    if kind == "pow2":
        return np.full(n, 1 << 20, np.uint64)
    if kind == "near_max":
        top = (1 << 63) // n - 1
        return rng.integers(top - 1000, top, n, dtype=np.uint64)
    if kind == "huge_spike":
        q = rng.integers(0, 1 << 10, n).astype(np.uint64)
        q[n // 2] = np.uint64(1 << 62)
        return q
    if kind == "sparse":
        q = np.zeros(n, np.uint64)
        pos = rng.choice(n, max(1, n // 50), replace=False)
        q[pos] = rng.integers(1, 1 << 40, len(pos), dtype=np.uint64)
        return q
    raise ValueError(kind)


@pytest.mark.parametrize("scheme", [1, 2])
@pytest.mark.parametrize("kind", ["tiny", "equal1", "pow2", "near_max",
                                  "huge_spike", "sparse"])
@pytest.mark.parametrize("n", [3, 130, 5000, 70001])
def test_fixed_point_resampler_boundaries(vc, port, scheme, kind, n):
    """CDF values on and next to the uniforms' grid: counts still bit-exact
    against the big-integer definition, and the engine advance unchanged."""
    import torch
    rng = np.random.default_rng(7 * n + scheme)
    q = _integer_weights(kind, n, rng)
    if int(q.sum()) == 0:
        q[0] = 1
    qi = [int(v) for v in q]
    assert sum(qi) < 1 << 63
    words = engine_words(port, n)
    ref = reference_counts(qi, scheme, words)
    r = vc.rng(vc.PHILOX4X32, key=list(KEY), ctr=list(CTR))
    rep = torch.zeros(n, dtype=torch.int32, device="cuda")
    idx = torch.zeros(n, dtype=torch.int32, device="cuda")
    vc.call("vsmc_cuda_resample_fixed", n, dev(q).data_ptr(), scheme,
            ctypes.byref(r), rep.data_ptr(), idx.data_ptr(), None)
    got = host(rep)
    assert np.array_equal(got, ref), int((got != ref).sum())
    want_idx = np.zeros(n, np.int32)
    port.vo_resample_trans_rep_index(n, n, P(ref), P(want_idx))
    assert np.array_equal(host(idx), want_idx)
    k = consumed(ref, scheme)
    total = 4 + k - 1
    assert r.index == total % 4 + 1


def test_fixed_point_resampler_rejects_zero_total(vc):
    """All-zero integer weights have no CDF: the call reports invalid
    weights instead of counting."""
    import torch
    n = 1000
    q = torch.zeros(n, dtype=torch.int64, device="cuda")
    r = vc.rng(vc.PHILOX4X32, key=list(KEY), ctr=list(CTR))
    rep = torch.zeros(n, dtype=torch.int32, device="cuda")
    rc = vc.lib().vsmc_cuda_resample_fixed(
        n, q.data_ptr(), 2, ctypes.byref(r), rep.data_ptr(), None, None)
    assert rc == vc.ERR_NONFINITE
