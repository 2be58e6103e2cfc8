"""vsmc_gb300 -- GB300 (sm_103a) backend for the vSMC particle-filter step.

The product is the C-ABI library ``libvsmc_cuda.so`` declared in
``include/vsmc_cuda.h``.  This module loads it with ctypes, declares every
prototype, and exposes thin Python wrappers that mirror the reference's C ABI
(``vsmc_rng_*``, ``vsmc_resample_*`` of include/vsmc/vsmc.h) and its
Sampler-level filter.  Arrays are device pointers (ints); callers usually pass
``tensor.data_ptr()`` of CUDA tensors.

There is no CPU fallback: if the CUDA library is missing or fails to load,
``lib()`` raises.
"""
import ctypes
import os

from . import build as _build

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = _build.LIB

VP = ctypes.c_void_p
SZ = ctypes.c_size_t
I32 = ctypes.c_int
U32 = ctypes.c_uint32
U64 = ctypes.c_uint64
F64 = ctypes.c_double
F32 = ctypes.c_float

# status codes (vsmc_cuda_status)
OK = 0
ERR_ARG = -1
ERR_SIZE = -2
ERR_NONFINITE = -3
ERR_TIMEOUT = -4
ERR_CUDA = -5
ERR_ALLOC = -6
ERR_INTERNAL = -7

PHILOX4X32 = 0
THREEFRY4X64 = 1

# vsmc::ResampleScheme order (internal/defines.hpp:57-64)
MULTINOMIAL = 0
STRATIFIED = 1
SYSTEMATIC = 2
RESIDUAL = 3
RESIDUAL_STRATIFIED = 4
RESIDUAL_SYSTEMATIC = 5
SCHEMES = {
    "multinomial": MULTINOMIAL,
    "stratified": STRATIFIED,
    "systematic": SYSTEMATIC,
    "residual": RESIDUAL,
    "residual_stratified": RESIDUAL_STRATIFIED,
    "residual_systematic": RESIDUAL_SYSTEMATIC,
}


class Rng(ctypes.Structure):
    """vsmc_cuda_rng: explicit CounterEngine state (kind, index, key, ctr)."""
    _fields_ = [("kind", ctypes.c_int32), ("index", ctypes.c_uint32),
                ("key", U64 * 4), ("ctr", U64 * 4)]


class CvModel(ctypes.Structure):
    """vsmc_cuda_cv_model."""
    _fields_ = [("dt", F64), ("sigma_a", F64), ("obs_scale", F64),
                ("nu", F64), ("sd_pos0", F64), ("sd_vel0", F64)]


class BearingsModel(ctypes.Structure):
    """vsmc_cuda_bearings_model."""
    _fields_ = [("dt", F64), ("q", F64), ("sigma_z", F64), ("x0", F64),
                ("y0", F64), ("vx0", F64), ("vy0", F64), ("sd_pos0", F64),
                ("sd_vel0", F64)]


def bearings_model():
    """The bearings-only benchmark model: dt 0.1, acceleration spectral
    density 1, bearing noise sd 0.005 rad, target starting near (10, 10)
    (position sd 1, velocity sd 1)."""
    return BearingsModel(0.1, 1.0, 0.005, 10.0, 10.0, 0.0, 0.0, 1.0, 1.0)


def default_model():
    """The benchmark tracking model: dt 0.1, acceleration sd 1, Student-t
    (nu 10, scale 0.5) observations, prior position sd 2, velocity sd 1."""
    return CvModel(0.1, 1.0, 0.5, 10.0, 2.0, 1.0)


class PfStepDesc(ctypes.Structure):
    """vsmc_cuda_pf_step_desc: the buffers of a filter's next step."""
    _fields_ = [("state_in", ctypes.c_void_p), ("state_out", ctypes.c_void_p),
                ("log_weight", ctypes.c_void_p), ("index", ctypes.c_void_p),
                ("sources", ctypes.c_void_p), ("partials", ctypes.c_void_p),
                ("scalars", ctypes.c_void_p), ("hist_mean", ctypes.c_void_p),
                ("hist_ess", ctypes.c_void_p), ("hist_logz", ctypes.c_void_p),
                ("hist_resampled", ctypes.c_void_p),
                ("n", ctypes.c_size_t), ("stride", ctypes.c_size_t),
                ("dim", ctypes.c_size_t), ("monitor_dim", ctypes.c_size_t),
                ("max_steps", ctypes.c_size_t), ("max_grid", ctypes.c_size_t),
                ("step", ctypes.c_size_t), ("seed", ctypes.c_uint32),
                ("threshold", ctypes.c_double), ("stream", ctypes.c_void_p),
                ("record_previous_mean", ctypes.c_int)]


class PfStatus(ctypes.Structure):
    """vsmc_cuda_pf_status: host view of a filter's device scalars."""
    _fields_ = [("ess", ctypes.c_double), ("log_evidence", ctypes.c_double),
                ("max_log_weight", ctypes.c_double),
                ("sum_weight", ctypes.c_double),
                ("mean", ctypes.c_double * 4), ("step", ctypes.c_size_t),
                ("resampled", ctypes.c_int), ("monitor_dim", ctypes.c_int)]


_RNGP = ctypes.POINTER(Rng)
_MODELP = ctypes.POINTER(CvModel)
_BMODELP = ctypes.POINTER(BearingsModel)

# name -> (restype, argtypes)
PROTOTYPES = {
    "vsmc_cuda_status_string": (ctypes.c_char_p, [I32]),
    "vsmc_cuda_last_cuda_error": (I32, []),
    "vsmc_cuda_version": (I32, []),
    "vsmc_cuda_rng_init": (I32, [_RNGP, I32, U64]),
    "vsmc_cuda_rng_set_key": (I32, [_RNGP, I32, VP]),
    "vsmc_cuda_rng_set_ctr": (I32, [_RNGP, I32, VP]),
    "vsmc_cuda_philox4x32_blocks": (I32, [VP, VP, SZ, VP, VP]),
    "vsmc_cuda_threefry4x64_blocks": (I32, [VP, VP, SZ, VP, VP]),
    "vsmc_cuda_rng_rand": (I32, [_RNGP, SZ, VP, VP]),
    "vsmc_cuda_rng_u01": (I32, [_RNGP, SZ, VP, VP]),
    "vsmc_cuda_rng_u01_f32": (I32, [_RNGP, SZ, VP, VP]),
    "vsmc_cuda_rng_normal": (I32, [_RNGP, SZ, VP, F64, F64, VP]),
    "vsmc_cuda_rng_normal_f32": (I32, [_RNGP, SZ, VP, F32, F32, VP]),
    "vsmc_cuda_rng_student_t": (I32, [_RNGP, SZ, VP, F64, VP]),
    "vsmc_cuda_normal_streams": (I32, [I32, VP, SZ, SZ, F64, F64, VP, VP]),
    "vsmc_cuda_student_t_streams": (I32, [I32, VP, SZ, SZ, F64, VP, VP]),
    "vsmc_cuda_u01_sorted": (I32, [SZ, VP, VP, VP]),
    "vsmc_cuda_u01_stratified": (I32, [SZ, VP, VP, VP]),
    "vsmc_cuda_u01_systematic": (I32, [SZ, F64, VP, VP]),
    "vsmc_cuda_sequential_sum": (I32, [SZ, VP, VP, VP, VP]),
    "vsmc_cuda_resample_trans_u01_rep": (I32, [SZ, SZ, VP, VP, VP, VP]),
    "vsmc_cuda_resample_trans_u01_index": (I32, [SZ, SZ, VP, VP, VP, VP]),
    "vsmc_cuda_resample_trans_rep_index": (I32, [SZ, SZ, VP, VP, VP]),
    "vsmc_cuda_resample_trans_index_rep": (I32, [SZ, SZ, VP, VP, VP]),
    "vsmc_cuda_resample_trans_residual": (
        I32, [SZ, SZ, VP, VP, VP, ctypes.POINTER(SZ), VP]),
    "vsmc_cuda_resample": (I32, [SZ, SZ, _RNGP, VP, VP, I32, VP]),
    "vsmc_cuda_resample_multinomial": (I32, [SZ, SZ, _RNGP, VP, VP, VP]),
    "vsmc_cuda_resample_stratified": (I32, [SZ, SZ, _RNGP, VP, VP, VP]),
    "vsmc_cuda_resample_systematic": (I32, [SZ, SZ, _RNGP, VP, VP, VP]),
    "vsmc_cuda_resample_residual": (I32, [SZ, SZ, _RNGP, VP, VP, VP]),
    "vsmc_cuda_resample_residual_stratified": (
        I32, [SZ, SZ, _RNGP, VP, VP, VP]),
    "vsmc_cuda_resample_residual_systematic": (
        I32, [SZ, SZ, _RNGP, VP, VP, VP]),
    "vsmc_cuda_resample_fixed": (I32, [SZ, VP, I32, _RNGP, VP, VP, VP]),
    "vsmc_cuda_resample_fixed_noalloc": (I32, [SZ, VP, I32, _RNGP, VP, VP,
                                               VP]),
    "vsmc_cuda_state_copy_f32": (I32, [SZ, SZ, VP, VP, VP]),
    "vsmc_cuda_state_copy_f64": (I32, [SZ, SZ, VP, VP, VP]),
    "vsmc_cuda_weight_set": (I32, [SZ, VP, VP, VP, VP]),
    "vsmc_cuda_weight_set_log": (I32, [SZ, VP, VP, VP, VP]),
    "vsmc_cuda_weight_add_log": (I32, [SZ, VP, VP, VP, VP]),
    "vsmc_cuda_weight_set_equal": (I32, [SZ, VP, VP, VP]),
    "vsmc_cuda_monitor_mean_f64": (I32, [SZ, SZ, VP, VP, VP, VP]),
    "vsmc_cuda_monitor_mean_f32": (I32, [SZ, SZ, VP, VP, VP, VP]),
    "vsmc_cuda_pf_create": (
        I32, [ctypes.POINTER(VP), SZ, I32, I32, F64, U32, _MODELP, SZ, VP]),
    "vsmc_cuda_pf_destroy": (I32, [VP]),
    "vsmc_cuda_pf_initialize": (I32, [VP, VP]),
    "vsmc_cuda_pf_iterate": (I32, [VP, VP]),
    "vsmc_cuda_pf_run_device": (I32, [VP, SZ, VP]),
    "vsmc_cuda_pf_run": (I32, [VP, SZ, VP, VP, VP, VP, VP]),
    "vsmc_cuda_pf_history": (I32, [VP, SZ, VP, VP, VP, VP]),
    "vsmc_cuda_pf_state": (I32, [VP, ctypes.POINTER(VP), ctypes.POINTER(VP)]),
    "vsmc_cuda_pf_stream": (I32, [VP, ctypes.POINTER(VP)]),
    "vsmc_cuda_pf_use_graph": (I32, [VP, I32]),
    "vsmc_cuda_pf_launch_step_kernel": (I32, [VP]),
    "vsmc_cuda_pf_create_model": (
        I32, [ctypes.POINTER(VP), SZ, SZ, SZ, I32, F64, U32, SZ, VP]),
    "vsmc_cuda_pf_step_desc_get": (I32, [VP, ctypes.POINTER(PfStepDesc)]),
    "vsmc_cuda_pf_status_enqueue": (I32, [VP]),
    "vsmc_cuda_pf_status_read": (I32, [VP, ctypes.POINTER(PfStatus)]),
    "vsmc_cuda_pf_step_advance": (I32, [VP]),
    "vsmc_cuda_pf_step_commit": (I32, [VP]),
    "vsmc_cuda_pf_reset": (I32, [VP]),
    "vsmc_cuda_pf_resample_now": (I32, [VP]),
    "vsmc_cuda_pf_set_equal": (I32, [VP]),
    "vsmc_cuda_pf_weight_log": (I32, [VP, VP, I32]),
    "vsmc_cuda_pf_get_status": (I32, [VP, ctypes.POINTER(PfStatus)]),
    "vsmc_cuda_batch_create": (
        I32, [ctypes.POINTER(VP), SZ, VP, VP, VP, VP, I32, F64, VP]),
    "vsmc_cuda_batch_create_bearings": (
        I32, [ctypes.POINTER(VP), SZ, VP, VP, VP, VP, VP, I32, F64, VP]),
    "vsmc_cuda_batch_destroy": (I32, [VP]),
    "vsmc_cuda_batch_set_schedule": (I32, [VP, U32]),
    "vsmc_cuda_batch_get_schedule": (I32, [VP, ctypes.POINTER(U32)]),
    "vsmc_cuda_batch_autotune_schedule": (I32, [VP, VP, I32, VP]),
    "vsmc_cuda_resample_index_trace": (I32, [SZ, SZ, VP, SZ, VP, VP]),
    "vsmc_cuda_resample_index_matrix": (I32, [SZ, SZ, VP, I32, VP, VP]),
    "vsmc_cuda_sampler_print": (I32, [SZ, SZ, VP, VP, SZ, ctypes.c_char_p,
                                      VP, SZ, VP, ctypes.c_char, VP, SZ,
                                      ctypes.POINTER(SZ)]),
    "vsmc_cuda_pf_record_genealogy": (I32, [VP, I32]),
    "vsmc_cuda_pf_set_mcmc": (I32, [VP, SZ, F64]),
    "vsmc_cuda_pf_mcmc_accepts": (I32, [VP, SZ, VP]),
    "vsmc_cuda_cv_mcmc_f32": (I32, [SZ, SZ, SZ, U32, _MODELP, VP, F64, VP, VP,
                                    VP, VP]),
    "vsmc_cuda_pf_genealogy": (I32, [VP, ctypes.POINTER(VP)]),
    "vsmc_cuda_pf_print": (I32, [VP, SZ, ctypes.c_char, VP, SZ,
                                 ctypes.POINTER(SZ)]),
    "vsmc_cuda_bearings_simulate": (I32, [U32, SZ, _BMODELP, VP, VP, VP]),
    "vsmc_cuda_mlp_sizes": (I32, [ctypes.POINTER(SZ), ctypes.POINTER(SZ)]),
    "vsmc_cuda_mlp_init": (I32, [U32, VP, VP]),
    "vsmc_cuda_mlp_pack": (I32, [VP, VP, VP]),
    "vsmc_cuda_mlp_forward": (I32, [VP, SZ, VP, VP, VP]),
    "vsmc_cuda_mlp_forward_tc": (I32, [VP, SZ, VP, VP, VP]),
    "vsmc_cuda_mlp_loss_grad": (I32, [VP, SZ, VP, VP, VP, VP, VP]),
    "vsmc_cuda_mlp_train": (I32, [_BMODELP, U32, SZ, SZ, SZ, SZ, F64, VP,
                                  VP, VP]),
    "vsmc_cuda_mlp_cloud_rows": (I32, [_BMODELP, U32, SZ, SZ, SZ, SZ, VP, VP,
                                       VP]),
    "vsmc_cuda_mlp_train_rows": (I32, [_BMODELP, U32, SZ, SZ, VP, VP, SZ, SZ,
                                       SZ, F64, VP, VP, VP]),
    "vsmc_cuda_bearings_move_f32": (I32, [SZ, SZ, U32, _BMODELP, F64, VP, VP,
                                          VP, VP]),
    "vsmc_cuda_batch_stream": (I32, [VP, ctypes.POINTER(VP)]),
    "vsmc_cuda_batch_simulate": (I32, [VP, VP, VP]),
    "vsmc_cuda_batch_run_device": (I32, [VP, VP]),
    "vsmc_cuda_batch_run": (I32, [VP, VP, VP, VP, VP, VP]),
    "vsmc_cuda_batch_history": (I32, [VP, VP, VP, VP, VP]),
    "vsmc_cuda_batch_set_shape": (I32, [VP, I32, I32]),
    "vsmc_cuda_batch_get_shape": (I32, [VP, ctypes.POINTER(I32),
                                        ctypes.POINTER(I32)]),
    "vsmc_cuda_batch_autotune": (I32, [VP, VP, I32, VP]),
    "vsmc_cuda_cv_move_f64": (I32, [SZ, SZ, U32, _MODELP, VP, VP, VP, VP]),
    "vsmc_cuda_cv_move_f32": (I32, [SZ, SZ, U32, _MODELP, VP, VP, VP, VP]),
    "vsmc_cuda_cv_simulate": (I32, [U32, SZ, _MODELP, VP, VP, VP]),
}

_LIB = None


class VsmcCudaError(RuntimeError):
    def __init__(self, status, where=""):
        msg = _status_text(status)
        if status == ERR_CUDA:
            try:
                msg += f", cudaError {lib().vsmc_cuda_last_cuda_error()}"
            except Exception:  # pragma: no cover
                pass
        super().__init__(f"{where}: status {status} ({msg})" if where else msg)
        self.status = status


def _status_text(status):
    try:
        return lib().vsmc_cuda_status_string(status).decode()
    except Exception:  # pragma: no cover - only when the library is broken
        return "unknown"


def lib(auto_build=True):
    """The loaded libvsmc_cuda (prototypes declared).  Raises if absent."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        if not auto_build:
            raise OSError(f"{LIB_PATH} is not built")
        _build.build()
    L = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(L, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    _LIB = L
    return L


def check(status, where=""):
    if status != OK:
        raise VsmcCudaError(status, where)
    return status


def call(name, *args):
    """Call an entry point and raise VsmcCudaError on a non-zero status."""
    return check(getattr(lib(), name)(*args), name)


def sampler_print(resampled, ess, mean, N, sep="\t", accept=None,
                  mon_name="pos"):
    """Sampler::print text from host histories (host-only code path)."""
    import numpy as np
    res = np.ascontiguousarray(resampled, dtype=np.int32)
    es = np.ascontiguousarray(ess, dtype=np.float64)
    mn = np.ascontiguousarray(mean, dtype=np.float64)
    T = len(es)
    nmon = mn.shape[1] if mn.ndim == 2 else 0
    acc = None
    nacc = 1
    if accept is not None:
        acc = np.ascontiguousarray(accept, dtype=np.uint64)
        nacc = acc.shape[1] if acc.ndim == 2 else 1
    n = SZ()
    args = [T, N, res.ctypes.data, es.ctypes.data, nmon, mon_name.encode(),
            mn.ctypes.data, nacc, acc.ctypes.data if acc is not None else None,
            sep.encode()]
    lib().vsmc_cuda_sampler_print(*args, None, 0, ctypes.byref(n))
    buf = ctypes.create_string_buffer(n.value + 1)
    call("vsmc_cuda_sampler_print", *args, buf, len(buf), ctypes.byref(n))
    return buf.value.decode()


def rng(kind=PHILOX4X32, seed=0, key=None, ctr=None):
    """A vsmc_cuda_rng placed like CounterEngine(seed), then key(k), ctr(c)."""
    r = Rng()
    call("vsmc_cuda_rng_init", ctypes.byref(r), kind, seed)
    if key is not None:
        k = (U64 * 4)(*[int(v) for v in key] + [0] * (4 - len(key)))
        call("vsmc_cuda_rng_set_key", ctypes.byref(r), len(key), k)
    if ctr is not None:
        c = (U64 * 4)(*[int(v) for v in ctr] + [0] * (4 - len(ctr)))
        call("vsmc_cuda_rng_set_ctr", ctypes.byref(r), len(ctr), c)
    return r


class FilterBatch:
    """Independent FP32 bootstrap filters stepped together
    (vsmc_cuda_batch): n, T, seeds are sequences, models a sequence of
    CvModel (default: the default model for every filter)."""

    def __init__(self, n, T, seeds, models=None, scheme=STRATIFIED,
                 threshold=0.5, stream=None, bearings=False, packed=None):
        """bearings=True: bearings-only filters (models: BearingsModel),
        with the learned proposal when packed (device pointer of the packed
        network) is given; observations are then one bearing per step."""
        import numpy as np
        self.n = np.ascontiguousarray(n, dtype=np.uint32)
        self.T = np.ascontiguousarray(T, dtype=np.uint32)
        self.seeds = np.ascontiguousarray(seeds, dtype=np.uint32)
        self.bearings = bearings
        self.obs_dim = 1 if bearings else 2
        nf = len(self.n)
        self.offsets = np.concatenate([[0], np.cumsum(self.T.astype(np.int64))])
        h = VP()
        if bearings:
            if models is None:
                models = [bearings_model() for _ in range(nf)]
            self.models = (BearingsModel * nf)(*models)
            call("vsmc_cuda_batch_create_bearings", ctypes.byref(h), nf,
                 self.n.ctypes.data, self.T.ctypes.data, self.models,
                 self.seeds.ctypes.data, packed, scheme, threshold, stream)
        else:
            if models is None:
                models = [default_model() for _ in range(nf)]
            self.models = (CvModel * nf)(*models)
            call("vsmc_cuda_batch_create", ctypes.byref(h), nf,
                 self.n.ctypes.data, self.T.ctypes.data, self.models,
                 self.seeds.ctypes.data, scheme, threshold, stream)
        self.handle = h

    @property
    def total_steps(self):
        return int(self.offsets[-1])

    def particle_steps(self):
        """Sum over the filters of particles x horizon."""
        return int(sum(int(a) * int(b) for a, b in zip(self.n, self.T)))

    def close(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            lib().vsmc_cuda_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):  # pragma: no cover - interpreter shutdown order
        try:
            self.close()
        except Exception:
            pass

    def stream(self):
        s = VP()
        call("vsmc_cuda_batch_stream", self.handle, ctypes.byref(s))
        return s.value

    def obs_len(self):
        """Doubles in the concatenated observation array."""
        return self.obs_dim * self.total_steps

    def simulate(self, obs_dev_ptr, truth_dev_ptr=None):
        call("vsmc_cuda_batch_simulate", self.handle, truth_dev_ptr,
             obs_dev_ptr)

    def run_device(self, obs_dev_ptr):
        call("vsmc_cuda_batch_run_device", self.handle, obs_dev_ptr)

    def _split(self, mean, ess, res, logz):
        out = []
        for f in range(len(self.n)):
            a, b = int(self.offsets[f]), int(self.offsets[f + 1])
            out.append({"mean": mean[a:b], "ess": ess[a:b],
                        "resampled": res[a:b], "logz": logz[a:b]})
        return out

    def history(self):
        """Per-filter histories of the last run (list of dicts)."""
        import numpy as np
        TT = self.total_steps
        mean = np.zeros((TT, 2))
        ess = np.zeros(TT)
        res = np.zeros(TT, dtype=np.int32)
        logz = np.zeros(TT)
        call("vsmc_cuda_batch_history", self.handle, mean.ctypes.data,
             ess.ctypes.data, res.ctypes.data, logz.ctypes.data)
        return self._split(mean, ess, res, logz)

    def run(self, obs):
        """Whole run through host buffers; obs: the concatenated
        observations (sum T x 2 positions, or sum T bearings)."""
        import numpy as np
        obs = np.ascontiguousarray(obs, dtype=np.float64)
        TT = self.total_steps
        mean = np.zeros((TT, 2))
        ess = np.zeros(TT)
        res = np.zeros(TT, dtype=np.int32)
        logz = np.zeros(TT)
        call("vsmc_cuda_batch_run", self.handle, obs.ctypes.data,
             mean.ctypes.data, ess.ctypes.data, res.ctypes.data,
             logz.ctypes.data)
        return self._split(mean, ess, res, logz)

    def set_shape(self, ppt, block):
        call("vsmc_cuda_batch_set_shape", self.handle, ppt, block)

    def shape(self):
        p, b = I32(), I32()
        call("vsmc_cuda_batch_get_shape", self.handle, ctypes.byref(p),
             ctypes.byref(b))
        return p.value, b.value

    def autotune(self, obs_dev_ptr, steps=50):
        import numpy as np
        ms = np.zeros(6, dtype=np.float32)
        call("vsmc_cuda_batch_autotune", self.handle, obs_dev_ptr, steps,
             ms.ctypes.data)
        return ms

    def set_schedule(self, min_chunk):
        call("vsmc_cuda_batch_set_schedule", self.handle, min_chunk)

    def schedule(self):
        c = U32()
        call("vsmc_cuda_batch_get_schedule", self.handle, ctypes.byref(c))
        return c.value

    def autotune_schedule(self, obs_dev_ptr, steps=50):
        import numpy as np
        ms = np.zeros(4, dtype=np.float32)
        call("vsmc_cuda_batch_autotune_schedule", self.handle, obs_dev_ptr,
             steps, ms.ctypes.data)
        return ms


class Proposal:
    """The proposal network's FP32 parameters and packed copy (device)."""

    def __init__(self, seed=0):
        import torch
        npar, npk = SZ(), SZ()
        call("vsmc_cuda_mlp_sizes", ctypes.byref(npar), ctypes.byref(npk))
        self.nparams, self.npacked = npar.value, npk.value
        self.params = torch.zeros(self.nparams, dtype=torch.float32,
                                  device="cuda")
        self.packed = torch.zeros(self.npacked, dtype=torch.int32,
                                  device="cuda")
        call("vsmc_cuda_mlp_init", seed, self.params.data_ptr(), None)
        self.pack()

    def pack(self):
        import torch
        call("vsmc_cuda_mlp_pack", self.params.data_ptr(),
             self.packed.data_ptr(), None)
        torch.cuda.synchronize()

    def train(self, model, seed, ntraj, T, batch, steps, lr, rows=None):
        """Adam on simulated trajectories, plus the extra training rows
        `rows` = (feat, nu) device tensors if given (for instance
        cloud_rows()); returns the minibatch losses."""
        import numpy as np
        losses = np.zeros(steps)
        if rows is None:
            call("vsmc_cuda_mlp_train", ctypes.byref(model), seed, ntraj, T,
                 batch, steps, lr, self.params.data_ptr(),
                 losses.ctypes.data, None)
        else:
            feat, nu = rows
            call("vsmc_cuda_mlp_train_rows", ctypes.byref(model), seed,
                 ntraj, T, feat.data_ptr(), nu.data_ptr(), nu.shape[0],
                 batch, steps, lr, self.params.data_ptr(),
                 losses.ctypes.data, None)
        self.pack()
        return losses

    def loss(self, feat_dev_ptr, nu_dev_ptr, B):
        """Mean loss on B rows (device arrays)."""
        import torch
        loss = torch.zeros(1, dtype=torch.float64, device="cuda")
        grad = torch.zeros(self.nparams, dtype=torch.float32, device="cuda")
        call("vsmc_cuda_mlp_loss_grad", self.packed.data_ptr(), B,
             feat_dev_ptr, nu_dev_ptr, loss.data_ptr(), grad.data_ptr(), None)
        return float(loss.cpu()[0])


class ParticleFilter:
    """A device-resident bootstrap filter (vsmc_cuda_pf) -- the Sampler<T>
    of the reference with the CUDA state / move / weight / monitor."""

    def __init__(self, n, precision=32, scheme=SYSTEMATIC, threshold=0.5,
                 seed=0, model=None, max_steps=256, stream=None):
        self.n = n
        self.precision = precision
        self.model = model if model is not None else default_model()
        h = VP()
        call("vsmc_cuda_pf_create", ctypes.byref(h), n, precision, scheme,
             threshold, seed, ctypes.byref(self.model), max_steps, stream)
        self.handle = h

    def close(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            lib().vsmc_cuda_pf_destroy(self.handle)
            self.handle = None

    def __del__(self):  # pragma: no cover - interpreter shutdown order
        try:
            self.close()
        except Exception:
            pass

    def launch_step_kernel(self):
        call("vsmc_cuda_pf_launch_step_kernel", self.handle)

    def use_graph(self, on):
        call("vsmc_cuda_pf_use_graph", self.handle, 1 if on else 0)

    def run(self, obs):
        """Whole run through host buffers; obs is a (T, 2) float64 array."""
        import numpy as np
        obs = np.ascontiguousarray(obs, dtype=np.float64)
        T = obs.shape[0]
        mean = np.zeros((T, 2))
        ess = np.zeros(T)
        res = np.zeros(T, dtype=np.int32)
        logz = np.zeros(T)
        call("vsmc_cuda_pf_run", self.handle, T, obs.ctypes.data,
             mean.ctypes.data, ess.ctypes.data, res.ctypes.data,
             logz.ctypes.data)
        return {"mean": mean, "ess": ess, "resampled": res, "logz": logz}

    def run_device(self, T, obs_dev_ptr):
        call("vsmc_cuda_pf_run_device", self.handle, T, obs_dev_ptr)

    def history(self, T):
        import numpy as np
        mean = np.zeros((T, 2))
        ess = np.zeros(T)
        res = np.zeros(T, dtype=np.int32)
        logz = np.zeros(T)
        call("vsmc_cuda_pf_history", self.handle, T, mean.ctypes.data,
             ess.ctypes.data, res.ctypes.data, logz.ctypes.data)
        return {"mean": mean, "ess": ess, "resampled": res, "logz": logz}

    def set_mcmc(self, sweeps, scale):
        call("vsmc_cuda_pf_set_mcmc", self.handle, sweeps, scale)

    def mcmc_accepts(self, T):
        import numpy as np
        out = np.zeros(T, dtype=np.uint32)
        call("vsmc_cuda_pf_mcmc_accepts", self.handle, T, out.ctypes.data)
        return out

    def record_genealogy(self, on=True):
        call("vsmc_cuda_pf_record_genealogy", self.handle, 1 if on else 0)

    def genealogy_ptr(self):
        p = VP()
        call("vsmc_cuda_pf_genealogy", self.handle, ctypes.byref(p))
        return p.value

    def print_tsv(self, T, sep="\t"):
        """Sampler::print text of the first T steps."""
        n = SZ()
        lib().vsmc_cuda_pf_print(self.handle, T, sep.encode(), None, 0,
                                 ctypes.byref(n))
        buf = ctypes.create_string_buffer(n.value + 1)
        call("vsmc_cuda_pf_print", self.handle, T, sep.encode(), buf,
             len(buf), ctypes.byref(n))
        return buf.value.decode()

    def state_ptrs(self):
        s, w = VP(), VP()
        call("vsmc_cuda_pf_state", self.handle, ctypes.byref(s),
             ctypes.byref(w))
        return s.value, w.value


def cloud_rows(model, seed, ntracks, particles, T, candidates):
    """Training rows from bootstrap-filter particle clouds
    (vsmc_cuda_mlp_cloud_rows): device tensors feat [rows, 6], nu [rows, 4]
    with rows = ntracks * particles * (T - 1)."""
    import torch
    rows = ntracks * particles * (T - 1)
    feat = torch.empty((rows, 6), dtype=torch.float32, device="cuda")
    nu = torch.empty((rows, 4), dtype=torch.float32, device="cuda")
    call("vsmc_cuda_mlp_cloud_rows", ctypes.byref(model), seed, ntracks,
         particles, T, candidates, feat.data_ptr(), nu.data_ptr(), None)
    torch.cuda.synchronize()
    return feat, nu
