"""vsmc_cuda_resample_fixed_noalloc against vsmc_cuda_resample_fixed: the
same replication counts, parent indices and engine advance on the same
integer weights, over two calls in a row (the second call must not see
anything the first left in the shared scratch array).  Integer outputs, so
the tolerance is zero."""
import ctypes

import numpy as np
import pytest

from conftest import dev, host

pytestmark = pytest.mark.gpu

MAX_N = 1 << 18  # VSMC_CUDA_RESAMPLE_FIXED_NOALLOC_MAX_N


def _weights(n, seed):
    rng = np.random.default_rng(seed)
    shift = 63 - int(np.ceil(np.log2(n)))
    lw = rng.normal(0, 3.0, n)
    w = np.exp(lw - lw.max())
    return np.floor(w * 2.0**shift).astype(np.uint64)


def _run(vc, name, n, q, scheme, r):
    import torch
    rep = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    idx = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    vc.call(name, n, q.data_ptr(), scheme, ctypes.byref(r), rep.data_ptr(),
            idx.data_ptr(), None)
    return host(rep), host(idx)


@pytest.mark.parametrize("scheme", [1, 2])
@pytest.mark.parametrize("n", [2, 1000, 65537, MAX_N])
def test_no_alloc_matches_allocating_entry(vc, scheme, n):
    ra = vc.rng(vc.PHILOX4X32, key=[99, 5], ctr=[0xFFFFFFFE, 1, 0, 0])
    rb = vc.rng(vc.PHILOX4X32, key=[99, 5], ctr=[0xFFFFFFFE, 1, 0, 0])
    for call in range(2):
        q = dev(_weights(n, 1000 * n + 10 * scheme + call))
        rep_a, idx_a = _run(vc, "vsmc_cuda_resample_fixed", n, q, scheme, ra)
        rep_b, idx_b = _run(vc, "vsmc_cuda_resample_fixed_noalloc", n, q,
                            scheme, rb)
        assert rep_a.sum() == n
        assert np.array_equal(rep_a, rep_b), (call, int((rep_a != rep_b).sum()))
        assert np.array_equal(idx_a, idx_b), (call, int((idx_a != idx_b).sum()))
        assert [int(v) for v in ra.ctr] == [int(v) for v in rb.ctr]
        assert ra.index == rb.index


def test_no_alloc_rejects_sizes_above_its_limit(vc):
    q = dev(np.ones(4, np.uint64))
    r = vc.rng(vc.PHILOX4X32, key=[1, 2], ctr=[0, 0, 0, 0])
    lib = vc.lib()
    st = lib.vsmc_cuda_resample_fixed_noalloc(MAX_N + 1, q.data_ptr(), 1,
                                              ctypes.byref(r), None, None, None)
    assert st == vc.ERR_SIZE
    assert [int(v) for v in r.ctr] == [0, 0, 0, 0]
