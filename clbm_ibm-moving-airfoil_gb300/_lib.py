"""ctypes binding of ``_build/libclbm_gb300.so`` (entry points of include/clbm_gb300.h).

The library is the only compute path: if it is missing, ``lib()`` raises instead of
falling back to anything else.
"""

import ctypes
import os

from . import build as _build

CLBM_OK = 0
CLBM_ERR_CUDA = 1
CLBM_ERR_ARG = 2
CLBM_ERR_DIVERGED = 3
CLBM_ERR_STATE = 4

STORAGE = {"f32": 0, "f16": 1, "bf16": 2}

EXPORTED = (
    "clbm_create", "clbm_destroy", "clbm_step", "clbm_step_dense_force",
    "clbm_step_host_force", "clbm_read_macro", "clbm_read_vorticity_slice",
    "clbm_read_populations", "clbm_write_populations", "clbm_check", "ibm_create",
    "ibm_destroy", "ibm_compute_force", "ibm_compute_force_motion", "ibm_read_forces",
    "ibm_read_markers", "ibm_read_force_history", "ibm_step_count", "clbm_run",
    "clbm_synchronize", "clbm_set_rho_floor", "clbm_selftest_wait_timeout", "clbm_stream", "clbm_profile_enable", "clbm_profile_read",
    "clbm_profile_read_split", "clbm_device_bytes", "clbm_kernel_variant", "clbm_binary_version",
    "clbm_state_bytes", "clbm_save_state", "clbm_load_state", "ibm_load_state",
    "clbm_bounds_checked", "clbm_selftest_bounds",
    "clbm_host_alloc", "clbm_host_free", "clbm_last_error", "ibm_force_sums_noalloc",
    "clbm_ensemble_create", "clbm_ensemble_run", "clbm_ensemble_stream",
    "clbm_ensemble_tuning", "clbm_ensemble_schedule", "clbm_ensemble_phase_times",
    "clbm_selftest_grid_barrier",
    "clbm_ensemble_destroy",
    "clbm_closure_layout", "clbm_closure_set", "clbm_trainer_create", "clbm_trainer_destroy",
    "clbm_trainer_capture", "clbm_trainer_read_slot", "clbm_trainer_extract", "clbm_trainer_count",
    "clbm_trainer_write_samples", "clbm_trainer_read_samples", "clbm_trainer_stats",
    "clbm_trainer_loss", "clbm_trainer_grad", "clbm_trainer_fit", "clbm_tc_selftest",
)


class CLBMError(RuntimeError):
    def __init__(self, code, message):
        super().__init__(f"[clbm error {code}] {message}")
        self.code = code


class DivergedError(CLBMError):
    pass


class Config(ctypes.Structure):
    """struct clbm_config"""
    _fields_ = [("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32),
                ("s_v", ctypes.c_double), ("s_e", ctypes.c_double),
                ("ux_in", ctypes.c_double), ("uy_in", ctypes.c_double),
                ("storage", ctypes.c_int32), ("device", ctypes.c_int32)]


class Motion(ctypes.Structure):
    """struct clbm_motion"""
    _fields_ = [(k, ctypes.c_double) for k in
                ("x0", "y0", "a_heave", "a_pitch", "phi_pitch", "aoa0", "w")]


_LIB = None


def lib_path():
    """The library the package loads: the bounds-checked build when CLBM_CHECK_BUILD=1."""
    return _build.LIB_CHECK if os.environ.get("CLBM_CHECK_BUILD") == "1" else _build.LIB


def lib():
    """Load the CUDA library (raises if it has not been built)."""
    global _LIB
    if _LIB is None:
        path = lib_path()
        if not os.path.exists(path):
            raise RuntimeError(
                f"CUDA library {path} is not built; run __graft_entry__.build() or "
                "python clbm_ibm-moving-airfoil_gb300/build.py")
        L = ctypes.CDLL(path)
        vp, P, i32, i64, d = (ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                              ctypes.c_int64, ctypes.c_double)
        pvp = ctypes.POINTER(ctypes.c_void_p)
        sig = {
            "clbm_create": [ctypes.POINTER(Config), pvp],
            "clbm_destroy": [vp],
            "clbm_step": [vp, vp],
            "clbm_step_dense_force": [vp, P, P, P],
            "clbm_step_host_force": [vp, P, P, P],
            "clbm_read_macro": [vp, P, P, P, P],
            "clbm_read_vorticity_slice": [vp, i32, P],
            "clbm_read_populations": [vp, P],
            "clbm_write_populations": [vp, P],
            "clbm_check": [vp, d, ctypes.POINTER(d), ctypes.POINTER(d), ctypes.POINTER(d),
                           ctypes.POINTER(i64)],
            "ibm_create": [vp, P, P, P, i32, pvp],
            "ibm_destroy": [vp],
            "ibm_compute_force": [vp, d, d, d, d, d, d],
            "ibm_compute_force_motion": [vp, ctypes.POINTER(Motion)],
            "ibm_read_forces": [vp, P, P, P],
            "ibm_read_markers": [vp, P],
            "ibm_read_force_history": [vp, i32, P],
            "ibm_step_count": [vp, ctypes.POINTER(i64)],
            "clbm_run": [vp, vp, ctypes.POINTER(Motion), i32, i32],
            "clbm_synchronize": [vp],
            "clbm_set_rho_floor": [vp, d],
            "clbm_stream": [vp, pvp],
            "clbm_selftest_wait_timeout": [vp, i32],
            "clbm_profile_enable": [vp, i32],
            "clbm_profile_read": [vp, ctypes.POINTER(d), ctypes.POINTER(i64), ctypes.POINTER(i64)],
            "clbm_profile_read_split": [vp, ctypes.POINTER(d), ctypes.POINTER(i64),
                                        ctypes.POINTER(d), ctypes.POINTER(i64)],
            "clbm_device_bytes": [vp, ctypes.POINTER(i64)],
            "clbm_kernel_variant": [vp, ctypes.POINTER(i32), ctypes.POINTER(ctypes.c_float)],
            "clbm_binary_version": [ctypes.POINTER(i32), ctypes.POINTER(i32)],
            "clbm_state_bytes": [vp, ctypes.POINTER(i64)],
            "clbm_bounds_checked": [ctypes.POINTER(i32)],
            "clbm_selftest_bounds": [vp],
            "clbm_save_state": [vp, vp, i64, ctypes.POINTER(i32)],
            "clbm_load_state": [vp, vp, i64, i32],
            "ibm_load_state": [vp, i64, P, i32],
            "clbm_host_alloc": [i64, pvp],
            "clbm_host_free": [vp],
            "ibm_force_sums_noalloc": [P, P, i32, i32, i32, P, P, i32, vp, P],
            "clbm_ensemble_create": [P, P, P, i32, pvp],
            "clbm_ensemble_run": [vp, i32, i32],
            "clbm_ensemble_stream": [vp, pvp],
            "clbm_ensemble_tuning": [vp, ctypes.POINTER(i32), ctypes.POINTER(i32),
                                     ctypes.POINTER(i64), ctypes.POINTER(ctypes.c_float),
                                     ctypes.POINTER(i32)],
            "clbm_ensemble_schedule": [vp, ctypes.POINTER(i32), ctypes.POINTER(i32)],
            "clbm_selftest_grid_barrier": [i32],
            "clbm_ensemble_phase_times": [vp, ctypes.POINTER(ctypes.c_double)],
            "clbm_ensemble_destroy": [vp],
            "clbm_closure_layout": [P],
            "clbm_closure_set": [vp, P],
            "clbm_trainer_create": [i32, vp, i64, pvp],
            "clbm_trainer_destroy": [vp],
            "clbm_trainer_capture": [vp, i32],
            "clbm_trainer_read_slot": [vp, i32, P],
            "clbm_trainer_extract": [vp, P, i64],
            "clbm_trainer_count": [vp, ctypes.POINTER(i64)],
            "clbm_trainer_write_samples": [vp, i64, i64, P],
            "clbm_trainer_read_samples": [vp, i64, i64, P],
            "clbm_trainer_stats": [vp, i64, i64, P],
            "clbm_trainer_loss": [vp, P, i64, i64, ctypes.c_float, ctypes.POINTER(d)],
            "clbm_trainer_grad": [vp, P, i64, i64, ctypes.c_float, P, ctypes.POINTER(d)],
            "clbm_trainer_fit": [vp, P, i64, i64, i32, i64, ctypes.c_float, ctypes.c_float,
                                 ctypes.c_uint64, P],
            "clbm_tc_selftest": [i32, P, P, P, i32, i32],
        }
        for name, args in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        L.clbm_last_error.argtypes = []
        L.clbm_last_error.restype = ctypes.c_char_p
        _LIB = L
    return _LIB


def check(rc):
    if rc != CLBM_OK:
        msg = lib().clbm_last_error().decode(errors="replace")
        if rc == CLBM_ERR_DIVERGED:
            raise DivergedError(rc, msg)
        raise CLBMError(rc, msg)
