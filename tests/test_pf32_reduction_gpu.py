"""The FP32 filter's weight reduction against an FP64 reduction of the same
log-weights at N = 2^24.

The fused step kernel sums exp(lw - m) and its square in FP32 within a
thread (about a hundred particles at N = 2^24), a warp and a block, then in
FP64 across blocks.  The reference keeps normalized FP64 weights and sums
them in FP64 (core/weight.hpp:208-230).  Here the device's ESS and
log-evidence increment of every step are compared with an FP64 reduction
(numpy, exact exp) of the very log-weights the kernel stored, with no
resampling in between (threshold 0), so only the reduction differs:

  ESS_t                 = (sum_i e_i)^2 / sum_i e_i^2,  e_i = exp(lw_i - max)
  log-evidence increment = logsumexp(lw_t) - logsumexp(lw_{t-1} - M_{t-1})

(the stored lw_t already carries the step's shift by the previous max
M_{t-1} in FP32).  Bars: 1e-5 relative on the ESS, 1e-5 absolute on the
increment."""
import ctypes

import numpy as np
import pytest


pytestmark = pytest.mark.gpu

N = 1 << 24
T = 8


def _lse(x):
    m = x.max()
    return m + np.log(np.exp(x - m).sum())


def test_fp32_block_reduction_against_fp64(vc):
    import torch
    obs_dev = torch.zeros(2 * T, dtype=torch.float64, device="cuda")
    m = vc.default_model()
    vc.call("vsmc_cuda_cv_simulate", 0, T, ctypes.byref(m),
            torch.zeros(4 * T, dtype=torch.float64, device="cuda").data_ptr(),
            obs_dev.data_ptr(), None)
    pf = vc.ParticleFilter(N, 32, vc.SYSTEMATIC, 0.0, seed=5, max_steps=T)
    L = vc.lib()
    prev_lw = None
    prev_M = None
    for t in range(T):
        ptr = obs_dev.data_ptr() + 16 * t
        if t == 0:
            vc.call("vsmc_cuda_pf_initialize", pf.handle, ctypes.c_void_p(ptr))
        else:
            vc.call("vsmc_cuda_pf_iterate", pf.handle, ctypes.c_void_p(ptr))
        st = vc.PfStatus()
        vc.check(L.vsmc_cuda_pf_get_status(pf.handle, ctypes.byref(st)))
        _, wptr = pf.state_ptrs()
        h = _download_f32(wptr, N)
        lw64 = h.astype(np.float64)
        e = np.exp(lw64 - lw64.max())
        ess64 = e.sum() ** 2 / (e * e).sum()
        assert abs(st.ess - ess64) / ess64 < 1e-5, (t, st.ess, ess64)
        hist = pf.history(t + 1)
        assert abs(hist["ess"][t] - ess64) / ess64 < 1e-5
        if t > 0:
            inc64 = _lse(lw64) - _lse(prev_lw - prev_M)
            inc = hist["logz"][t] - hist["logz"][t - 1]
            assert abs(inc - inc64) < 1e-5, (t, inc, inc64)
        else:
            inc64 = _lse(lw64) - np.log(N)
            assert abs(hist["logz"][0] - inc64) < 1e-5
        prev_lw = lw64
        prev_M = float(np.float32(st.max_log_weight))
    pf.close()


def _download_f32(dev_ptr, n):
    """n floats from a raw device address (cudaMemcpy through ctypes)."""
    import torch
    out = np.empty(n, np.float32)
    cudart = None
    for name in ("libcudart.so.13", "libcudart.so"):
        try:
            cudart = ctypes.CDLL(name)  # the runtime libvsmc_cuda loaded
            break
        except OSError:
            continue
    assert cudart is not None
    torch.cuda.synchronize()
    rc = cudart.cudaMemcpy(ctypes.c_void_p(out.ctypes.data),
                           ctypes.c_void_p(dev_ptr), ctypes.c_size_t(4 * n),
                           ctypes.c_int(2))
    assert rc == 0, rc
    return out
