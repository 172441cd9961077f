"""ctypes binding of libvlagpu.so (declared in include/vlagpu.h).

The library is the only compute path of this package: if it is not built, or
no CUDA device is present, every operator raises.  There is no CPU fallback.
"""

from __future__ import annotations

import ctypes as C
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libvlagpu.so")

VG_OK = 0
VG_ERR_ARG = 1
VG_ERR_CUDA = 2
VG_ERR_UNSUPPORTED = 3
VG_ERR_NUMERIC = 4
VG_ERR_TIMEOUT = 5
VG_ERR_STATE = 6

VG_F64 = 0
VG_F32_DELTA_F = 1
VG_COLL_NONE, VG_COLL_LB, VG_COLL_DG = 0, 1, 2
VG_LEAPFROG, VG_PEFRL, VG_H_SIXTH = 0, 1, 2
VG_ENV_TANH, VG_ENV_SIN2 = 0, 1

DP = C.POINTER(C.c_double)


class VgPulse(C.Structure):
    _fields_ = [("k0", C.c_double), ("w0", C.c_double), ("a0", C.c_double),
                ("t_L", C.c_double), ("t_R", C.c_double), ("t_wL", C.c_double),
                ("t_wR", C.c_double), ("envelope", C.c_int32), ("reserved", C.c_int32)]


class VgRunDesc(C.Structure):
    _fields_ = [("nx", C.c_int32), ("nv", C.c_int32), ("precision", C.c_int32),
                ("collision", C.c_int32), ("integrator", C.c_int32), ("n_pulses", C.c_int32),
                ("dt", C.c_double), ("nu", C.c_double), ("dx", C.c_double), ("dv", C.c_double),
                ("dv_sq", C.c_double),
                ("x", DP), ("v", DP), ("kx", DP), ("kv", DP), ("one_over_kx", DP),
                ("v_pow", DP), ("pulses", C.POINTER(VgPulse)), ("f_background", DP)]


class VgHistory(C.Structure):
    _fields_ = [("nt", C.c_int32), ("store_all", C.c_int32), ("n_modes", C.c_int32),
                ("n_slots", C.c_int32), ("fields", C.c_void_p * 8), ("series", C.c_void_p * 7),
                ("stored_f", C.c_void_p)]


class VgSweepRun(C.Structure):
    _fields_ = [("nx", C.c_int32), ("nv", C.c_int32), ("k", C.c_double), ("amplitude", C.c_double),
                ("nu", C.c_double)]


class VgSweepDesc(C.Structure):
    _fields_ = [("n_runs", C.c_int32), ("collision", C.c_int32), ("vmax", C.c_double), ("dt", C.c_double),
                ("runs", C.POINTER(VgSweepRun))]


class VgCorrBatch(C.Structure):
    _fields_ = [("g", C.c_void_p), ("g_prev", C.c_void_p), ("row_feat", C.c_void_p), ("target", C.c_void_p),
                ("rows", C.c_int32), ("group_rows", C.c_int32)]


class VgProfEntry(C.Structure):
    _fields_ = [("name", C.c_char * 32), ("launches", C.c_int64), ("total_ms", C.c_double),
                ("bytes_per_launch", C.c_double)]


EXPORTS = {
    # name: (restype, argtypes)
    "vg_version": (C.c_int, []),
    "vg_last_error": (C.c_char_p, []),
    "vg_plan_create": (C.c_int, [C.POINTER(VgRunDesc), C.POINTER(C.c_void_p)]),
    "vg_plan_destroy": (C.c_int, [C.c_void_p]),
    "vg_edfdv": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_void_p]),
    "vg_vdfdx": (C.c_int, [C.c_void_p, C.c_void_p, C.c_double, C.c_void_p]),
    "vg_vdfdx_sl": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_void_p]),
    "vg_edfdv_sl": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_void_p]),
    "vg_edfdv_cd2": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_void_p]),
    "vg_charge_density": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "vg_poisson": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "vg_field_solve": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "vg_collision_step": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "vg_storage_step": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                  C.POINTER(VgHistory), C.c_int32, C.c_void_p]),
    "vg_driver": (C.c_int, [C.c_void_p, C.c_double, C.c_void_p, C.c_void_p]),
    "vg_run_steps": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(VgHistory),
                               C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32,
                               C.c_void_p]),
    "vg_field_solve_noalloc": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_double, C.c_void_p,
                                         C.c_void_p, C.c_void_p, C.c_void_p]),
    "vg_batch_create": (C.c_int, [C.POINTER(VgRunDesc), C.c_int32, C.POINTER(C.c_void_p)]),
    "vg_batch_destroy": (C.c_int, [C.c_void_p]),
    "vg_batch_sizes": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "vg_batch_run_steps": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p,
                                     C.c_int32, C.c_int32, C.c_int32, C.c_void_p]),
    "vg_batch_profile_enable": (C.c_int, [C.c_void_p, C.c_int32]),
    "vg_batch_profile_read": (C.c_int, [C.c_void_p, C.POINTER(VgProfEntry), C.c_int32, C.POINTER(C.c_int32)]),
    "vg_sweep_create": (C.c_int, [C.POINTER(VgSweepDesc), C.POINTER(C.c_void_p)]),
    "vg_sweep_destroy": (C.c_int, [C.c_void_p]),
    "vg_sweep_sizes": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "vg_sweep_x_offsets": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "vg_sweep_reset": (C.c_int, [C.c_void_p, C.c_void_p]),
    "vg_sweep_run_steps": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32,
                                     C.c_int32, C.c_void_p]),
    "vg_sweep_read_run": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]),
    "vg_sweep_get_state": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "vg_sweep_set_state": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "vg_sweep_state_ptr": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]),
    "vg_sweep_damping": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_double, C.c_double, C.c_double,
                                   C.c_void_p, C.c_void_p, C.c_void_p]),
    "vg_sweep_status": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "vg_sweep_set_step_events": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.c_int32]),
    "vg_sweep_set_wait_limit": (C.c_int, [C.c_void_p, C.c_int64]),
    "vg_sweep_inject_lost_tiles": (C.c_int, [C.c_void_p, C.c_int32]),
    "vg_plan_status": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "vg_batch_status": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "vg_sweep_profile_enable": (C.c_int, [C.c_void_p, C.c_int32]),
    "vg_sweep_profile_read": (C.c_int, [C.c_void_p, C.POINTER(VgProfEntry), C.c_int32, C.POINTER(C.c_int32)]),
    "vg_profile_enable": (C.c_int, [C.c_void_p, C.c_int32]),
    "vg_profile_read": (C.c_int, [C.c_void_p, C.POINTER(VgProfEntry), C.c_int32,
                                  C.POINTER(C.c_int32)]),
    "vg_corr_num_params": (C.c_int, []),
    "vg_corr_create": (C.c_int, [C.c_int32, C.c_int32, C.c_float, C.c_float, C.c_void_p, C.POINTER(C.c_void_p)]),
    "vg_corr_destroy": (C.c_int, [C.c_void_p]),
    "vg_corr_set_tau": (C.c_int, [C.c_void_p, C.c_float]),
    "vg_corr_get_params": (C.c_int, [C.c_void_p, C.c_void_p]),
    "vg_corr_set_params": (C.c_int, [C.c_void_p, C.c_void_p]),
    "vg_corr_apply": (C.c_int, [C.c_void_p, C.POINTER(VgCorrBatch), C.c_void_p, C.c_void_p]),
    "vg_corr_set_engine": (C.c_int, [C.c_void_p, C.c_int32]),
    "vg_corr_status": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "vg_corr_loss": (C.c_int, [C.c_void_p, C.POINTER(VgCorrBatch), C.POINTER(C.c_double), C.c_void_p]),
    "vg_corr_gradients": (C.c_int, [C.c_void_p, C.POINTER(VgCorrBatch), C.c_void_p, C.POINTER(C.c_double),
                                    C.c_void_p]),
    "vg_corr_train_step": (C.c_int, [C.c_void_p, C.POINTER(VgCorrBatch), C.c_float, C.POINTER(C.c_double),
                                     C.c_void_p]),
}

_lib = None
_lock = threading.Lock()


def load(path: str | None = None):
    """Load (once) and return the library; raises if it is not built."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise RuntimeError(
                "libvlagpu.so is not built (%s); run `python -m vlapy_gb300.build` "
                "(or __graft_entry__.build()) on a machine with nvcc" % p)
        lib = C.CDLL(p)
        for name, (res, args) in EXPORTS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


class VlagpuError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("vlagpu error %d: %s" % (status, msg))
        self.status = status


def check(status: int, what: str = ""):
    """Raise the reference-style exception for a non-zero status."""
    if status == VG_OK:
        return
    msg = load().vg_last_error().decode(errors="replace")
    if what:
        msg = what + ": " + msg
    if status == VG_ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    if status == VG_ERR_ARG:
        raise ValueError(msg)
    raise VlagpuError(status, msg)
