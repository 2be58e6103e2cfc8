"""The C ABI calls that the C++ backend classes (include/vsmc_cuda_backend.hpp)
make under the reference's Sampler<T>, in the order Sampler<T> makes them,
against the oracle's FP64 filter.  The classes themselves need the
reference's headers and are compiled against them by test_backend_cpu.py;
this test runs the same device calls where those headers are absent.

Sampler<T>::initialize / iterate (core/sampler.hpp:443-476, 735-785):
init (InitializeCV: vsmc_cuda_cv_move_f64 at t = 0, WeightCUDA::set_log) or
move (MoveCV: vsmc_cuda_cv_move_f64 at t, WeightCUDA::add_log), then
Particle::resample (core/particle.hpp:170-197): when ESS < threshold * N,
StateCUDA::copy(N, nullptr) runs vsmc_cuda_resample, rep -> index and the
in-place state copy, and the weights are set equal; then the monitor
(MonitorMeanCUDA: vsmc_cuda_monitor_mean_f64)."""
import ctypes

import numpy as np
import pytest

from conftest import P, host

pytestmark = pytest.mark.gpu


def _obs(port, T, seed=0):
    from oracle.binding import default_model
    tr = np.zeros(4 * T)
    ob = np.zeros(2 * T)
    port.vo_pf_simulate(seed, T, ctypes.byref(default_model()), P(tr), P(ob))
    return ob.reshape(T, 2)


@pytest.mark.parametrize("scheme", [1, 2])
def test_sampler_call_sequence_matches_oracle_filter(vc, port, scheme):
    import torch
    from oracle.binding import default_model
    N, T, seed, threshold = 1 << 14, 50, 5, 0.5
    obs = np.ascontiguousarray(_obs(port, T))
    model = vc.default_model()
    f64 = dict(dtype=torch.float64, device="cuda")
    i32 = dict(dtype=torch.int32, device="cuda")
    state = torch.zeros(4 * N, **f64)
    ll = torch.zeros(N, **f64)
    W = torch.zeros(N, **f64)
    ess_dev = torch.zeros(1, **f64)
    rep = torch.zeros(N, **i32)
    idx = torch.zeros(N, **i32)
    out = torch.zeros(2, **f64)
    # StateCUDA::resample_scheme: Philox4x32 keyed {0, seed}, counter
    # {0, 0, 1, 0}
    rng = vc.rng(vc.PHILOX4X32, key=[0, seed], ctr=[0, 0, 1, 0])
    mean = np.zeros((T, 2))
    ess = np.zeros(T)
    res = np.zeros(T, np.int32)
    for t in range(T):
        ob = np.ascontiguousarray(obs[t])
        vc.call("vsmc_cuda_cv_move_f64", N, t, seed, ctypes.byref(model),
                P(ob), state.data_ptr(), ll.data_ptr(), None)
        if t == 0:
            vc.call("vsmc_cuda_weight_set_log", N, ll.data_ptr(),
                    W.data_ptr(), ess_dev.data_ptr(), None)
        else:
            vc.call("vsmc_cuda_weight_add_log", N, ll.data_ptr(),
                    W.data_ptr(), ess_dev.data_ptr(), None)
        ess[t] = float(host(ess_dev)[0])
        if ess[t] < threshold * N:
            res[t] = 1
            vc.call("vsmc_cuda_resample", N, N, ctypes.byref(rng),
                    W.data_ptr(), rep.data_ptr(), scheme, None)
            vc.call("vsmc_cuda_resample_trans_rep_index", N, N,
                    rep.data_ptr(), idx.data_ptr(), None)
            vc.call("vsmc_cuda_state_copy_f64", N, 4, idx.data_ptr(),
                    state.data_ptr(), None)
            vc.call("vsmc_cuda_weight_set_equal", N, W.data_ptr(),
                    ess_dev.data_ptr(), None)
        vc.call("vsmc_cuda_monitor_mean_f64", N, 2, state.data_ptr(),
                W.data_ptr(), out.data_ptr(), None)
        mean[t] = host(out)
    # the oracle's FP64 filter: the reference's arithmetic step for step
    om, oe = np.zeros(2 * T), np.zeros(T)
    orr, oz = np.zeros(T, np.int32), np.zeros(T)
    port.vo_pf_run(64, N, T, seed, scheme, threshold,
                   ctypes.byref(default_model()), P(obs), 0, P(om), P(oe),
                   P(orr), P(oz))
    assert np.array_equal(res, orr)
    np.testing.assert_allclose(ess, oe, rtol=1e-8)
    np.testing.assert_allclose(mean, om.reshape(T, 2), rtol=1e-8, atol=1e-8)
