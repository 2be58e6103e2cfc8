"""Device lineage tracing against the reference's ResampleIndex fixtures and
the oracle, and the FP32 filter's genealogy recording."""
import ctypes
import os

import numpy as np
import pytest

from conftest import GOLDEN, P, dev, host

pytestmark = pytest.mark.gpu


def _trace_matrix(vc, rows):
    import torch
    iters, N = rows.shape
    d = dev(np.ascontiguousarray(rows, np.int32))
    tr = torch.zeros((iters, N), dtype=torch.int32, device="cuda")
    for it in range(iters):
        vc.call("vsmc_cuda_resample_index_trace", N, iters, d.data_ptr(), it,
                tr[it].data_ptr(), None)
    mats = []
    for layout in (0, 1):
        m = torch.zeros(N * iters, dtype=torch.int32, device="cuda")
        vc.call("vsmc_cuda_resample_index_matrix", N, iters, d.data_ptr(),
                layout, m.data_ptr(), None)
        mats.append(host(m))
    return host(tr).ravel(), mats


def test_device_index_matches_reference_fixtures(vc):
    g = np.load(os.path.join(GOLDEN, "genealogy.npz"))
    for si in range(int(g["nsizes"][0])):
        tr, mats = _trace_matrix(vc, g[f"rows{si}"])
        assert np.array_equal(tr, g[f"trace{si}"])
        for layout in (0, 1):
            assert np.array_equal(mats[layout], g[f"matrix{si}_{layout}"])


def test_device_index_matches_oracle_large(vc, port):
    rng = np.random.default_rng(1)
    N, iters = 10007, 41
    rows = np.sort(rng.integers(0, N, (iters, N)), axis=1).astype(np.int32)
    rows[::5] = np.arange(N)
    tr, mats = _trace_matrix(vc, rows)
    ref_tr = np.zeros((iters, N), np.int32)
    for it in range(iters):
        port.vo_resample_index_trace(N, iters, P(rows), it, P(ref_tr[it]))
    assert np.array_equal(tr, ref_tr.ravel())
    for layout in (0, 1):
        m = np.zeros(N * iters, np.int32)
        port.vo_resample_index_matrix(N, iters, P(rows), layout, P(m))
        assert np.array_equal(mats[layout], m)


def test_device_index_rejects_out_of_range_rows(vc):
    import torch
    rows = dev(np.array([[0, 5, 1]], np.int32).repeat(2, axis=0))
    out = torch.zeros(6, dtype=torch.int32, device="cuda")
    st = vc.lib().vsmc_cuda_resample_index_matrix(3, 2, rows.data_ptr(), 0,
                                                  out.data_ptr(), None)
    assert st == vc.ERR_ARG


def test_filter_genealogy_and_print(vc, port):
    import torch
    from oracle.binding import default_model
    T, n = 40, 5000
    tr = np.zeros(4 * T)
    ob = np.zeros(2 * T)
    port.vo_pf_simulate(1, T, ctypes.byref(default_model()), P(tr), P(ob))
    obs = ob.reshape(T, 2)
    plain = vc.ParticleFilter(n, 32, 1, 0.5, seed=4, max_steps=T)
    ref = plain.run(obs)
    plain.close()
    pf = vc.ParticleFilter(n, 32, 1, 0.5, seed=4, max_steps=T)
    pf.record_genealogy(True)
    got = pf.run(obs)
    # recording does not change the filter
    for k in ("mean", "ess", "resampled", "logz"):
        assert np.array_equal(got[k], ref[k]), k
    rows_ptr = pf.genealogy_ptr()
    rows = torch.zeros((T, n), dtype=torch.int32, device="cuda")
    # device-to-device copy of the recorded rows
    vc.call("vsmc_cuda_resample_index_trace", n, 1, rows_ptr, 0,
            rows[0].data_ptr(), None)  # row 0 (a one-row history traces to itself)
    rows_np = np.zeros((T, n), np.int32)
    for t in range(T):
        vc.call("vsmc_cuda_resample_index_trace", n, 1,
                ctypes.c_void_p(rows_ptr + 4 * n * t), 0,
                rows[t].data_ptr(), None)
    rows_np[:] = host(rows)
    ident = np.arange(n)
    for t in range(T):
        r = rows_np[t]
        if got["resampled"][t]:
            assert (r >= 0).all() and (r < n).all()
            kept = np.unique(r)
            assert np.array_equal(r[kept], kept)  # parents keep their slot
            assert not np.array_equal(r, ident)
        else:
            assert np.array_equal(r, ident)
    # the lineage of the recorded rows on the device equals the oracle's
    rows.copy_(torch.from_numpy(rows_np).cuda())
    m = torch.zeros(T * n, dtype=torch.int32, device="cuda")
    vc.call("vsmc_cuda_resample_index_matrix", n, T, rows.data_ptr(), 1,
            m.data_ptr(), None)
    ref_m = np.zeros(T * n, np.int32)
    port.vo_resample_index_matrix(n, T, P(rows_np), 1, P(ref_m))
    assert np.array_equal(host(m), ref_m)
    # summary text: the filter's histories through the Sampler::print writer
    text = pf.print_tsv(T)
    assert text == vc.sampler_print(got["resampled"], got["ess"], got["mean"],
                                    n)
    assert text.splitlines()[0] == "\t".join(
        ["Size", "Resampled", "Accept.0", "ESS", "pos.0", "pos.1", ""])
    pf.close()
