"""Loader of the CUDA library ``libssgpu.so`` (the C ABI of include/ssgpu.h).

The library is built in tree by ``build.py``.  There is no CPU fallback: if the
library cannot be built or loaded, every entry point raises.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libssgpu.so")

# every symbol that include/ssgpu.h declares
EXPORTS = [
    "ss_create", "ss_destroy", "ss_init", "ss_init_distribution", "ss_resume", "ss_do_timestep", "ss_run", "ss_noise", "ss_step_host",
    "ss_synchronize",
    "ss_get_particles", "ss_get_distribution", "ss_get_counts", "ss_get_flow_field", "ss_get_magnetic_field",
    "ss_get_flow_complex", "ss_get_magnetic_complex", "ss_get_timestep", "ss_output_begin", "ss_output_wait",
    "ss_output_query", "ss_host_alloc", "ss_host_free", "ss_mean_flow_field",
    "ss_mean_magnetic_field", "ss_langevin", "ss_set_resort", "ss_profile_enable", "ss_profile_read", "ss_launch_count",
    "ss_sample_distribution_noalloc", "ss_ensemble_create", "ss_ensemble_destroy", "ss_ensemble_init",
    "ss_ensemble_autotune", "ss_ensemble_set_config", "ss_ensemble_run", "ss_ensemble_synchronize", "ss_ensemble_get_particles",
    "ss_ensemble_get_counts", "ss_ensemble_get_flow_field", "ss_ensemble_info", "ss_dn_conv32", "ss_dn_create",
    "ss_dn_destroy", "ss_dn_info", "ss_dn_set_loss", "ss_dn_get_params", "ss_dn_set_params", "ss_dn_forward", "ss_dn_train",
    "ss_dn_gradients", "ss_dn_sample_histogram", "ss_set_denoiser", "ss_fp64_rate", "ss_last_error", "ss_version",
]

SS_OK = 0
SS_ERR_INVALID_ARGUMENT = 1
SS_ERR_CUDA = 2
SS_ERR_CUFFT = 3
SS_ERR_STATE = 4
SS_ERR_PARTICLE_COUNT = 5
SS_ERR_RANGE = 6

FLAG_QUASI2D = 1
FLAG_ALWAYS_MAGNETIC = 2
FLAG_NO_SORT = 4
FLAG_NO_GRAPH = 8
FLAG_MIXED = 16
FLAG_TRILINEAR = 32
FLAG_TRILINEAR_ZFROMY = 64
FLAG_FIXED64 = 128
FLAG_F32X2 = 256

NUM_STAGES = 8
STAGES = ["contract", "fft_forward", "kspace", "fft_inverse", "table", "update", "sort", "other"]


class SsError(RuntimeError):
    """A non-zero status from the C ABI."""

    def __init__(self, code, msg):
        super().__init__(f"[ssgpu status {code}] {msg}")
        self.code = code


class Grid(ctypes.Structure):
    _fields_ = [("x", ctypes.c_uint64), ("y", ctypes.c_uint64), ("z", ctypes.c_uint64),
                ("phi", ctypes.c_uint64), ("theta", ctypes.c_uint64)]


class Box(ctypes.Structure):
    _fields_ = [("x", ctypes.c_double), ("y", ctypes.c_double), ("z", ctypes.c_double)]


class Params(ctypes.Structure):
    _fields_ = [
        ("timestep", ctypes.c_double), ("trans_diffusion", ctypes.c_double), ("rot_diffusion", ctypes.c_double),
        ("stress_active", ctypes.c_double), ("stress_magnetic", ctypes.c_double), ("shape", ctypes.c_double),
        ("magnetic_drag", ctypes.c_double), ("hydro_screening", ctypes.c_double),
        ("volume_exclusion", ctypes.c_double), ("magnetic_reorientation", ctypes.c_double),
        ("magnetic_dipole_dipole", ctypes.c_double), ("number_of_particles", ctypes.c_uint64),
        ("seed", ctypes.c_uint64),
    ]


class LangevinArgs(ctypes.Structure):
    _fields_ = [
        ("flow", ctypes.c_double * 3), ("drag", ctypes.c_double), ("gradb", ctypes.c_double * 9),
        ("reorientation", ctypes.c_double), ("b", ctypes.c_double * 3), ("vort", ctypes.c_double * 9),
        ("shape", ctypes.c_double), ("strain", ctypes.c_double * 9), ("dt", ctypes.c_double),
        ("xi", ctypes.c_double * 3), ("diff", ctypes.c_double), ("axis_angle", ctypes.c_double),
        ("rotate_angle", ctypes.c_double), ("box_x", ctypes.c_double), ("box_y", ctypes.c_double),
        ("box_z", ctypes.c_double),
    ]


_lib = None


def load(build_if_missing=True):
    """Load libssgpu.so (building it first when absent); raises on failure."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise OSError(f"{LIB_PATH} is missing; run __graft_entry__.build()")
        from . import build as _build
        _build.build()
    L = ctypes.CDLL(LIB_PATH)
    vp, dp, u64, u32 = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_uint64, ctypes.c_uint32
    u64p = ctypes.POINTER(ctypes.c_uint64)
    ci = ctypes.c_int
    sig = {
        "ss_create": [ctypes.POINTER(Grid), ctypes.POINTER(Box), ctypes.POINTER(Params), u32, vp,
                      ctypes.POINTER(vp)],
        "ss_destroy": [vp],
        "ss_init": [vp, dp, u64],
        "ss_resume": [vp, dp, u64, u64],
        "ss_init_distribution": [vp, u32],
        "ss_do_timestep": [vp, dp, u64p],
        "ss_run": [vp, u64, u64p],
        "ss_noise": [vp, u64, dp],
        "ss_step_host": [vp, dp, dp, u64, u64p],
        "ss_synchronize": [vp],
        "ss_get_particles": [vp, dp, u64],
        "ss_get_distribution": [vp, dp],
        "ss_get_counts": [vp, ctypes.POINTER(ctypes.c_uint32)],
        "ss_get_flow_field": [vp, dp],
        "ss_get_magnetic_field": [vp, dp],
        "ss_get_flow_complex": [vp, dp, dp],
        "ss_get_magnetic_complex": [vp, dp, dp],
        "ss_get_timestep": [vp, u64p],
        "ss_output_begin": [vp, ci, dp, dp, dp, dp, u64],
        "ss_output_wait": [vp, ci],
        "ss_output_query": [vp, ci, ctypes.POINTER(ci)],
        "ss_host_alloc": [u64, ctypes.POINTER(vp)],
        "ss_host_free": [vp],
        "ss_mean_flow_field": [vp, ctypes.c_double, dp, dp, dp],
        "ss_mean_magnetic_field": [vp, dp, dp, dp],
        "ss_langevin": [dp, u64, u32, ctypes.POINTER(LangevinArgs), dp],
        "ss_set_resort": [vp, u32],
        "ss_profile_enable": [vp, ci],
        "ss_profile_read": [vp, dp, u64p],
        "ss_launch_count": [vp, u64p],
        "ss_fp64_rate": [dp],
        "ss_sample_distribution_noalloc": [ctypes.POINTER(Grid), ctypes.POINTER(Box), vp, u64, vp, vp],
        "ss_ensemble_create": [ctypes.POINTER(Grid), ctypes.POINTER(Box), ctypes.POINTER(Params), u32, u32, vp,
                               ctypes.POINTER(vp)],
        "ss_ensemble_destroy": [vp],
        "ss_ensemble_init": [vp, dp, u64],
        "ss_ensemble_autotune": [vp, ctypes.POINTER(ctypes.c_uint32)],
        "ss_ensemble_set_config": [vp, ctypes.POINTER(ctypes.c_uint32)],
        "ss_ensemble_run": [vp, u64],
        "ss_ensemble_synchronize": [vp],
        "ss_ensemble_get_particles": [vp, u32, dp],
        "ss_ensemble_get_counts": [vp, u32, ctypes.POINTER(ctypes.c_uint32)],
        "ss_ensemble_get_flow_field": [vp, u32, dp],
        "ss_ensemble_info": [vp, u64p, ctypes.POINTER(ctypes.c_uint32), u64p],
        "ss_dn_conv32": [vp, vp, vp, vp, vp, u32, u32, u32, u32, vp],
        "ss_dn_create": [u32, u32, u32, u64, vp, ctypes.POINTER(vp)],
        "ss_dn_destroy": [vp],
        "ss_dn_set_loss": [vp, ctypes.c_float],
        "ss_dn_info": [vp, u64p, u64p],
        "ss_dn_get_params": [vp, ctypes.POINTER(ctypes.c_float), u64],
        "ss_dn_set_params": [vp, ctypes.POINTER(ctypes.c_float), u64],
        "ss_dn_forward": [vp, vp, vp],
        "ss_dn_train": [vp, vp, vp, u32, ctypes.c_float, dp],
        "ss_dn_gradients": [vp, vp, vp, u32, ctypes.POINTER(ctypes.c_float), u64, dp],
        "ss_set_denoiser": [vp, vp],
        "ss_dn_sample_histogram": [u32, u32, u32, u64, ctypes.c_double, ctypes.c_double, u32, u64, vp, vp],
        "ss_last_error": [vp, ctypes.c_char_p, ctypes.c_size_t],
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = ci
    L.ss_version.argtypes = []
    L.ss_version.restype = ctypes.c_char_p
    _lib = L
    return L


def last_error(ctx=None):
    buf = ctypes.create_string_buffer(1024)
    load().ss_last_error(ctx, buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc, ctx=None):
    if rc != SS_OK:
        raise SsError(rc, last_error(ctx))
