"""Genealogy and summary text on the CPU: the oracle's ResampleIndex
restatement against the reference's own index traces and matrices, and the
library's Sampler::print writer (host code, no GPU) against the reference's
print of the same run, byte for byte."""
import os

import numpy as np

from conftest import GOLDEN, P


def _g():
    return np.load(os.path.join(GOLDEN, "genealogy.npz"))


def test_oracle_resample_index_matches_reference(port):
    g = _g()
    for si in range(int(g["nsizes"][0])):
        rows = np.ascontiguousarray(g[f"rows{si}"])
        iters, N = rows.shape
        tr = np.zeros((iters, N), np.int32)
        for it in range(iters):
            port.vo_resample_index_trace(N, iters, P(rows), it, P(tr[it]))
        assert np.array_equal(tr.ravel(), g[f"trace{si}"]), si
        for layout in (0, 1):
            m = np.zeros(N * iters, np.int32)
            port.vo_resample_index_matrix(N, iters, P(rows), layout, P(m))
            assert np.array_equal(m, g[f"matrix{si}_{layout}"]), (si, layout)


def test_sampler_print_matches_reference_text():
    import vsmc_gb300 as vc
    g = _g()
    text = vc.sampler_print(g["tsv_res"], g["tsv_ess"], g["tsv_mean"],
                            int(g["tsv_N"][0]))
    assert text == bytes(g["tsv"]).decode()


def test_sampler_print_edge_cases():
    import vsmc_gb300 as vc
    assert vc.sampler_print([], [], np.zeros((0, 2)), 10) == ""
    t = vc.sampler_print([1], [float("nan")], [[1e-7, 123456789.0]], 3,
                         sep=",", accept=[2])
    assert t == "Size,Resampled,Accept.0,ESS,pos.0,pos.1,\n3,1,2,nan,1e-07,1.23457e+08,\n"
