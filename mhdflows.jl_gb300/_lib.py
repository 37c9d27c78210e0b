"""ctypes binding of ``include/mhdgb.h`` (the C ABI a Julia ``ccall`` wrapper binds the same way).

The library must exist (built in-tree by ``build.py``); there is no fallback: a missing or
unloadable library raises immediately.
"""
from __future__ import annotations

import ctypes as C
import os
import re

from . import build as _build

HEADER = os.path.join(_build.INCLUDE, "mhdgb.h")

MHD_OK = 0
MHD_ERR_INVALID = 1
MHD_ERR_CUDA = 2
MHD_ERR_OOM = 3
MHD_ERR_NONFINITE = 4
MHD_ERR_STATE = 5
MHD_RK4 = 0
MHD_LSRK4 = 1
MHD_DIV_U = 1
MHD_DIV_B = 2
MHD_PREC_FP32 = 0
MHD_PREC_SPLIT_FP16 = 1
MHD_PREC_SPLIT_BF16 = 2
MHD_PREC_SPLIT_TF32 = 3
MHD_TUNE_FORCE = 1
MHD_TUNE_NO_FILE = 2


class MHDError(RuntimeError):
    """Raised for a non-zero status of the C ABI (the reference raises Julia ``error(...)``)."""

    def __init__(self, code: int, msg: str):
        super().__init__(msg)
        self.code = code


class MhdParams(C.Structure):
    _fields_ = [
        ("n", C.c_int),
        ("L", C.c_double),
        ("nu", C.c_double),
        ("eta", C.c_double),
        ("nnu", C.c_int),
        ("neta", C.c_int),
        ("dt", C.c_double),
        ("scheme", C.c_int),
        ("precision", C.c_int),
        ("device", C.c_int),
        ("hydro_only", C.c_int),
        ("vp", C.c_int),
    ]


class MhdServerParams(C.Structure):
    _fields_ = [
        ("budget_bytes", C.c_double),
        ("steps_per_tick", C.c_int),
        ("scheme", C.c_int),
        ("device", C.c_int),
        ("keep_states", C.c_int),
        ("capacity", C.c_int * 8),
    ]


class MhdRequest(C.Structure):
    _fields_ = [
        ("n", C.c_int),
        ("L", C.c_double),
        ("nu", C.c_double),
        ("eta", C.c_double),
        ("dt", C.c_double),
        ("steps", C.c_longlong),
        ("sol", C.c_void_p),
    ]


_SIGS = {
    "mhd_create": (C.c_int, [C.POINTER(MhdParams), C.POINTER(C.c_void_p)]),
    "mhd_destroy": (C.c_int, [C.c_void_p]),
    "mhd_supported_n": (C.c_int, [C.c_int]),
    "mhd_kept_modes": (C.c_int, [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "mhd_set_state": (C.c_int, [C.c_void_p, C.c_void_p]),
    "mhd_get_state": (C.c_int, [C.c_void_p, C.c_void_p]),
    "mhd_set_physical": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "mhd_get_physical": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "mhd_step": (C.c_int, [C.c_void_p, C.c_int]),
    "mhd_compute_rhs": (C.c_int, [C.c_void_p, C.c_void_p]),
    "mhd_get_clock": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_longlong), C.POINTER(C.c_double)]),
    "mhd_set_clock": (C.c_int, [C.c_void_p, C.c_double, C.c_longlong, C.c_double]),
    "mhd_diagnostics": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.c_int]),
    "mhd_synchronize": (C.c_int, [C.c_void_p]),
    "mhd_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "mhd_get_stream": (C.c_void_p, [C.c_void_p]),
    "mhd_memory_bytes": (C.c_int, [C.c_void_p, C.POINTER(C.c_longlong)]),
    "mhd_footprint_bytes": (C.c_int, [C.POINTER(MhdParams), C.POINTER(C.c_longlong)]),
    "mhd_host_alloc": (C.c_int, [C.c_size_t, C.POINTER(C.c_void_p)]),
    "mhd_host_free": (C.c_int, [C.c_void_p]),
    "mhd_profile_enable": (C.c_int, [C.c_void_p, C.c_int]),
    "mhd_profile_read": (C.c_int, [C.c_void_p, C.POINTER(C.c_longlong), C.POINTER(C.c_double), C.c_int]),
    "mhd_kernel_class_name": (C.c_char_p, [C.c_int]),
    "mhd_kernel_class_count": (C.c_int, []),
    "mhd_kernel_class_bytes": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double)]),
    "mhd_time_steps": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double)]),
    "mhd_step_timed": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double)]),
    "mhd_batch_create": (C.c_int, [C.POINTER(MhdParams), C.c_int, C.POINTER(C.c_void_p)]),
    "mhd_batch_add": (C.c_int, [C.c_void_p, C.c_double, C.c_double, C.c_double, C.POINTER(C.c_int)]),
    "mhd_batch_remove": (C.c_int, [C.c_void_p, C.c_int]),
    "mhd_batch_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "mhd_slot_bytes": (C.c_int, [C.POINTER(MhdParams), C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]),
    "mhd_slot_set_state": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "mhd_slot_get_state": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "mhd_set_state_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "mhd_get_state_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "mhd_slot_set_state_device": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "mhd_slot_get_state_device": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "mhd_slot_set_physical": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p]),
    "mhd_slot_get_physical": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p]),
    "mhd_slot_diagnostics": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double), C.c_int]),
    "mhd_slot_get_clock": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_longlong), C.POINTER(C.c_double)]),
    "mhd_slot_set_clock": (C.c_int, [C.c_void_p, C.c_int, C.c_double, C.c_longlong, C.c_double]),
    "mhd_ensemble_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.POINTER(C.c_void_p)]),
    "mhd_ensemble_step": (C.c_int, [C.c_void_p, C.c_int]),
    "mhd_ensemble_destroy": (C.c_int, [C.c_void_p]),
    "mhd_set_cfl": (C.c_int, [C.c_void_p, C.c_int, C.c_double]),
    "mhd_diagnostics_noalloc": (C.c_int, [C.c_void_p, C.c_int, C.c_double, C.c_void_p, C.c_void_p]),
    "mhd_set_forcing": (C.c_int, [C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_double, C.c_ulonglong]),
    "mhd_slot_set_forcing": (C.c_int, [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                       C.c_ulonglong]),
    "mhd_get_forcing": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "mhd_set_vp": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "mhd_slot_set_vp": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "mhd_div_correct": (C.c_int, [C.c_void_p, C.c_int]),
    "mhd_slot_div_correct": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "mhd_set_div_correction": (C.c_int, [C.c_void_p, C.c_int]),
    "mhd_set_diag_history": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "mhd_get_diag_history": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.POINTER(C.c_int)]),
    "mhd_check_guards": (C.c_int, [C.c_void_p, C.POINTER(C.c_longlong)]),
    "mhd_server_create": (C.c_int, [C.POINTER(MhdServerParams), C.POINTER(C.c_void_p)]),
    "mhd_server_destroy": (C.c_int, [C.c_void_p]),
    "mhd_server_submit": (C.c_int, [C.c_void_p, C.POINTER(MhdRequest), C.POINTER(C.c_longlong)]),
    "mhd_server_tick": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "mhd_server_poll": (C.c_int, [C.c_void_p, C.c_longlong, C.POINTER(C.c_int), C.POINTER(C.c_longlong)]),
    "mhd_server_result": (C.c_int, [C.c_void_p, C.c_longlong, C.c_void_p, C.c_void_p]),
    "mhd_server_cancel": (C.c_int, [C.c_void_p, C.c_longlong]),
    "mhd_server_memory": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "mhd_check_bounded_wait": (C.c_int, [C.c_int, C.c_double, C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    "mhd_autotune": (C.c_int, [C.c_void_p, C.c_int]),
    "mhd_variant_count": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int)]),
    "mhd_variant_name": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_char_p, C.c_int]),
    "mhd_select_variant": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "mhd_last_error": (C.c_char_p, []),
}

_lib = None


def header_functions(path: str = HEADER):
    """Names of the functions declared in the C header."""
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mhd_[a-z0-9_]+)\s*\(", text)))


def load(path: str | None = None):
    """Load libmhdgb.so (building it first if the sources are newer) and bind every symbol."""
    global _lib
    if _lib is not None:
        return _lib
    if path is None:
        path = _build.build()
    if not os.path.exists(path):
        raise MHDError(MHD_ERR_STATE, f"CUDA library missing: {path} (run build())")
    lib = C.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc: int):
    if rc != MHD_OK:
        msg = _lib.mhd_last_error().decode() if _lib is not None else "error"
        raise MHDError(rc, msg)
    return rc
