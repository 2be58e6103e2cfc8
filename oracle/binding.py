"""ctypes loader for the oracle libraries (test infrastructure only).

    port()  -> oracle/_build/libvsmc_oracle.so, the C restatement (built with
               `make -C oracle port` on first use; works on x86 and Arm)
    ref()   -> oracle/_ref/libvsmcref.so, the reference compiled from its own
               sources, or None where it is not built (the GPU host has no
               reference tree)

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline arm use this.
"""
import ctypes
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
PORT = os.path.join(HERE, "_build", "libvsmc_oracle.so")
REF = os.path.join(HERE, "_ref", "libvsmcref.so")

VP = ctypes.c_void_p
SZ = ctypes.c_size_t
I32 = ctypes.c_int
U32 = ctypes.c_uint32
F64 = ctypes.c_double
F32 = ctypes.c_float


class Model(ctypes.Structure):
    _fields_ = [("dt", F64), ("sigma_a", F64), ("obs_scale", F64),
                ("nu", F64), ("sd_pos0", F64), ("sd_vel0", F64)]


def default_model():
    return Model(0.1, 1.0, 0.5, 10.0, 2.0, 1.0)


_MP = ctypes.POINTER(Model)


class BModel(ctypes.Structure):
    """vo_bmodel: the bearings-only tracking model."""
    _fields_ = [("dt", F64), ("q", F64), ("sigma_z", F64), ("x0", F64),
                ("y0", F64), ("vx0", F64), ("vy0", F64), ("sd_pos0", F64),
                ("sd_vel0", F64)]


def bearings_model():
    return BModel(0.1, 1.0, 0.005, 10.0, 10.0, 0.0, 0.0, 1.0, 1.0)


_BMP = ctypes.POINTER(BModel)

PORT_PROTOTYPES = {
    "vo_philox4x32_words": (None, [VP, VP, SZ, VP, I32]),
    "vo_threefry4x64_words": (None, [VP, VP, SZ, VP, I32]),
    "vo_u01_u32_f64_n": (None, [I32, SZ, VP, VP]),
    "vo_u01_u32_f32_n": (None, [I32, SZ, VP, VP]),
    "vo_u01_u64_f64_n": (None, [I32, SZ, VP, VP]),
    "vo_u01_dist_f64": (None, [I32, VP, VP, SZ, VP, I32]),
    "vo_u01_dist_f32": (None, [I32, VP, VP, SZ, VP, I32]),
    "vo_normal_f64": (None, [I32, VP, VP, SZ, F64, F64, VP, I32]),
    "vo_normal_f32": (None, [I32, VP, VP, SZ, F32, F32, VP, I32]),
    "vo_student_t_f64": (None, [I32, VP, VP, SZ, F64, VP]),
    "vo_student_t_batch_f64": (None, [I32, VP, VP, SZ, SZ, F64, VP, VP, VP]),
    "vo_u01_sequence": (None, [I32, SZ, VP, VP, VP, VP]),
    "vo_u01_sorted": (None, [SZ, VP, VP]),
    "vo_u01_stratified": (None, [SZ, VP, VP]),
    "vo_u01_systematic": (None, [SZ, F64, VP]),
    "vo_resample_trans_u01_rep": (None, [SZ, SZ, VP, VP, VP]),
    "vo_resample_trans_u01_index": (None, [SZ, SZ, VP, VP, VP]),
    "vo_resample_trans_rep_index": (None, [SZ, SZ, VP, VP]),
    "vo_resample_trans_index_rep": (None, [SZ, SZ, VP, VP]),
    "vo_resample_trans_residual": (SZ, [SZ, SZ, VP, VP, VP]),
    "vo_resample_words": (None, [I32, SZ, SZ, VP, VP, VP, VP, VP]),
    "vo_state_copy_f32": (None, [SZ, VP, VP]),
    "vo_state_copy_f64": (None, [SZ, VP, VP]),
    "vo_weight_set_log": (F64, [SZ, VP, VP]),
    "vo_weight_add_log": (F64, [SZ, VP, VP, VP]),
    "vo_weight_set": (F64, [SZ, VP, VP]),
    "vo_pf_simulate": (None, [U32, SZ, _MP, VP, VP]),
    "vo_pf_run_replay": (I32, [I32, SZ, SZ, U32, _MP, VP, VP, VP, VP, VP, VP]),
    "vo_pf_run": (I32, [I32, SZ, SZ, U32, I32, F64, _MP, VP, I32, VP, VP, VP,
                        VP]),
    "vo_pf_move_f64": (None, [SZ, SZ, U32, _MP, VP, VP, VP]),
    "vo_pf_move_f32": (None, [SZ, SZ, U32, _MP, VP, VP, VP]),
    "vo_pf_init_f64": (None, [SZ, U32, _MP, VP, VP, VP]),
    "vo_pf_init_f32": (None, [SZ, U32, _MP, VP, VP, VP]),
    "vo_student_t_norm_const": (F64, [F64, F64]),
    "vo_bearings_simulate": (None, [U32, SZ, _BMP, VP, VP]),
    "vo_bearings_move_f32": (None, [SZ, SZ, U32, _BMP, F64, VP, VP, VP]),
    "vo_mlp_forward": (None, [VP, SZ, VP, VP]),
    "vo_mlp_loss_grad": (None, [VP, SZ, VP, VP, VP, VP]),
    "vo_mlp_set_rounding": (None, [I32]),
    "vo_resample_index_trace": (None, [SZ, SZ, VP, SZ, VP]),
    "vo_cv_mcmc_f32": (None, [SZ, SZ, SZ, U32, _MP, VP, F64, VP, VP, VP, VP]),
    "vo_resample_index_matrix": (None, [SZ, SZ, VP, I32, VP]),
    "vo_bearings_pf_run": (I32, [I32, SZ, SZ, U32, I32, F64, _BMP, VP, VP,
                                 I32, VP, VP, VP, VP]),
    "vo_engine_run": (None, [I32, VP, VP, SZ, I32, SZ, F64, F64, VP, VP,
                             VP]),
}

REF_PROTOTYPES = {
    "ref_philox4x32_words": (None, [VP, VP, SZ, VP, I32]),
    "ref_threefry4x64_words": (None, [VP, VP, SZ, VP, I32]),
    "ref_u01_u32_f64": (None, [I32, SZ, VP, VP]),
    "ref_u01_u32_f32": (None, [I32, SZ, VP, VP]),
    "ref_u01_u64_f64": (None, [I32, SZ, VP, VP]),
    "ref_u01_dist_f64": (None, [I32, VP, VP, SZ, VP, I32]),
    "ref_u01_dist_f32": (None, [I32, VP, VP, SZ, VP, I32]),
    "ref_normal_f64": (None, [I32, VP, VP, SZ, F64, F64, VP, I32]),
    "ref_normal_f32": (None, [I32, VP, VP, SZ, F32, F32, VP, I32]),
    "ref_student_t_f64": (None, [I32, VP, VP, SZ, F64, VP, I32]),
    "ref_u01_sequence": (None, [I32, SZ, VP, VP, VP, VP]),
    "ref_resample": (None, [I32, SZ, SZ, VP, VP, VP, VP, VP]),
    "ref_state_copy_f32": (None, [SZ, VP, VP]),
    "ref_state_copy_f64": (None, [SZ, VP, VP]),
    "ref_weight_set_log": (F64, [SZ, VP, VP]),
    "ref_weight_add_log": (F64, [SZ, VP, VP, VP]),
    "ref_weight_set": (F64, [SZ, VP, VP]),
    "ref_pf_run": (I32, [I32, SZ, SZ, U32, I32, F64, I32, F64, F64, F64, F64,
                         F64, F64, VP, VP, VP, VP, VP]),
    "ref_pf_print": (SZ, [SZ, SZ, U32, I32, F64, F64, F64, F64, F64, F64,
                          F64, VP, VP, VP, VP, VP, ctypes.c_char_p, SZ]),
    "ref_resample_index": (None, [SZ, SZ, VP, I32, VP, VP]),
    "ref_pf_simulate": (None, [U32, SZ, F64, F64, F64, F64, F64, F64, VP,
                               VP]),
    "vsmc_resample_trans_u01_rep": (None, [I32, I32, VP, VP, VP]),
    "vsmc_resample_trans_u01_index": (None, [I32, I32, VP, VP, VP]),
    "vsmc_resample_trans_rep_index": (None, [I32, I32, VP, VP]),
    "vsmc_resample_trans_index_rep": (None, [I32, I32, VP, VP]),
    "vsmc_resample_trans_residual": (I32, [I32, I32, VP, VP, VP]),
    "vsmc_rng_u01_sorted": (None, [I32, VP, VP]),
    "vsmc_rng_u01_stratified": (None, [I32, VP, VP]),
    "vsmc_rng_u01_systematic": (None, [I32, F64, VP]),
}

_port = None
_ref = None


def _declare(lib, table):
    for name, (res, args) in table.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


def build_port():
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return PORT


# Where this recipe reads the reference tree: VSMC_REF_ROOT, else the
# read-only checkout of the build container.  The GPU host has neither.
_REF_CHECKOUT = "/root/reference"


def ref_root():
    """The reference source tree (VSMC_REF_ROOT or the build container's
    checkout), or None where it is absent."""
    root = os.environ.get("VSMC_REF_ROOT") or _REF_CHECKOUT
    if os.path.isdir(os.path.join(root, "include", "vsmc")):
        return root
    return None


def build_ref():
    """Build the reference library if the reference tree is present."""
    root = ref_root()
    if root is None:
        return None
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_ROOT={root}"],
                   check=True)
    return REF


def port():
    global _port
    if _port is None:
        build_port()
        _port = _declare(ctypes.CDLL(PORT), PORT_PROTOTYPES)
    return _port


def ref():
    global _ref
    if _ref is None:
        if not os.path.exists(REF):
            return None
        _ref = _declare(ctypes.CDLL(REF), REF_PROTOTYPES)
    return _ref
