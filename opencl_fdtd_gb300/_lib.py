"""
ctypes binding of the C ABI declared in include/fdtd_gb300.h.

The structures below mirror the header field for field; tests compare their sizes and
offsets with what a C compiler reports for the header. Loading fails loudly when the
library is not built: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

c_i32, c_i64, c_f64, c_vp = ctypes.c_int32, ctypes.c_int64, ctypes.c_double, ctypes.c_void_p

FDTD_OK = 0
FDTD_ERR_INVALID = -1
FDTD_ERR_UNSUPPORTED = -2
FDTD_ERR_CUDA = -3
FDTD_ERR_WATCHDOG = -4
FDTD_ERR_NONFINITE = -5
FDTD_F32 = 0
FDTD_F64 = 1
FDTD_TUNE_XCHUNK = 1
FDTD_TUNE_SLAB = 2
FDTD_TUNE_FUSED_ROWS = 3
FDTD_TUNE_FUSED_XCHUNK = 4
FDTD_TUNE_HS_XCHUNK = 5
FDTD_TUNE_HS_PREFETCH = 6
FDTD_TUNE_TIMING = 7
FDTD_TUNE_FUSED_STAGES = 8
FDTD_TUNE_FUSED_TMA = 9
FDTD_TUNE_FUSED_SHAPE = 10
FDTD_TUNE_HS_REVERSE = 11
FDTD_TUNE_HS_DFT = 13
FDTD_TUNE_PDL = 14
FDTD_TUNE_E_FORM = 15
FDTD_GET_LAST_RUN_PATH = 100
FDTD_GET_STEP_ROWS = 101
FDTD_GET_STEP_XCHUNK = 102
FDTD_GET_STEP_STAGES = 103
FDTD_GET_STEP_THREADS = 104
FDTD_GET_STEP_SHAPE = 105
FDTD_GET_HS_XCHUNK_USED = 106
FDTD_PATH_NONE = 0
FDTD_PATH_PER_UPDATE = 1
FDTD_PATH_HS = 2
FDTD_PATH_ONEPASS = 3


class FdtdPmlDesc(ctypes.Structure):
    _fields_ = [("axis", c_i32), ("polarity", c_i32), ("thickness", c_i32), ("_pad", c_i32),
                ("p0e", c_vp), ("p1e", c_vp), ("p2e", c_vp),
                ("p0h", c_vp), ("p1h", c_vp), ("p2h", c_vp)]


class FdtdBlochDesc(ctypes.Structure):
    _fields_ = [("axis", c_i32), ("_pad", c_i32), ("real", c_f64), ("imag", c_f64)]


class FdtdDesc(ctypes.Structure):
    _fields_ = [("shape", c_i64 * 3), ("dtype", c_i32), ("uniform", c_i32),
                ("dt", c_f64), ("dx", c_f64),
                ("n_pml", c_i32), ("n_bloch", c_i32),
                ("pml", FdtdPmlDesc * 6), ("bloch", FdtdBlochDesc * 3),
                ("do_poynting", c_i32), ("do_fieldsrc", c_i32), ("has_mu", c_i32), ("_pad", c_i32)]


_PSI = (c_vp * 2) * 6


class FdtdBuffers(ctypes.Structure):
    _fields_ = [("E", c_vp), ("H", c_vp), ("F", c_vp), ("G", c_vp),
                ("eps", c_vp), ("mu", c_vp), ("S", c_vp), ("oS", c_vp),
                ("Jr", c_vp), ("Ji", c_vp),
                ("psi_e", _PSI), ("psi_h", _PSI), ("psi_f", _PSI), ("psi_g", _PSI),
                ("inv_de", c_vp * 3), ("inv_dh", c_vp * 3),
                ("ce", c_vp), ("cm", c_vp),
                ("E2", c_vp), ("H2", c_vp), ("psi_e2", _PSI), ("psi_h2", _PSI)]


class FdtdPointSources(ctypes.Structure):
    _fields_ = [("n", c_i32), ("_pad", c_i32), ("index", c_vp), ("values", c_vp)]


class FdtdDftMonitor(ctypes.Structure):
    _fields_ = [("n_points", c_i32), ("n_freq", c_i32), ("index", c_vp), ("omega", c_vp),
                ("accum", c_vp), ("series", c_vp), ("step", c_i64), ("series_row", c_i64)]


FDTD_STORE_F32, FDTD_STORE_BF16, FDTD_STORE_F16, FDTD_STORE_BF16U = 0, 1, 2, 3
FDTD_BATCH_MAX_SRC, FDTD_BATCH_MAX_MON = 4, 8
FDTD_BATCH_PERSISTENT, FDTD_BATCH_LAUNCHES = 0, 1


class FdtdBatchFace(ctypes.Structure):
    _fields_ = [("axis", c_i32), ("polarity", c_i32), ("thickness", c_i32), ("_pad", c_i32),
                ("tab_e", c_vp * 3), ("tab_h", c_vp * 3), ("psi_e", c_vp * 2), ("psi_h", c_vp * 2)]


class FdtdBatchVariant(ctypes.Structure):
    _fields_ = [("shape", c_i32 * 3), ("n_pml", c_i32), ("dt", c_f64), ("dx", c_f64),
                ("pml", FdtdBatchFace * 6), ("E", c_vp), ("H", c_vp), ("ce", c_vp),
                ("e_exp", c_vp), ("h_exp", c_vp), ("n_src", c_i32), ("n_mon", c_i32),
                ("src_index", c_i64 * FDTD_BATCH_MAX_SRC), ("src_values", c_vp),
                ("mon_index", c_i64 * FDTD_BATCH_MAX_MON), ("series", c_vp)]


# (name, restype, argtypes) of every entry point in include/fdtd_gb300.h
_P = ctypes.POINTER
SIGNATURES = [
    ("fdtd_abi_version", c_i32, []),
    ("fdtd_last_error", ctypes.c_char_p, []),
    ("fdtd_plan_create", c_i32, [_P(FdtdDesc), _P(c_vp)]),
    ("fdtd_plan_destroy", c_i32, [c_vp]),
    ("fdtd_plan_tune", c_i32, [c_vp, c_i32, c_i32]),
    ("fdtd_plan_get", c_i32, [c_vp, c_i32, _P(c_i32)]),
    ("fdtd_prepare", c_i32, [c_vp, _P(FdtdBuffers), c_vp]),
    ("fdtd_update_e", c_i32, [c_vp, _P(FdtdBuffers), c_vp]),
    ("fdtd_update_h", c_i32, [c_vp, _P(FdtdBuffers), c_vp]),
    ("fdtd_update_s", c_i32, [c_vp, _P(FdtdBuffers), c_vp]),
    ("fdtd_update_f", c_i32, [c_vp, _P(FdtdBuffers), c_vp]),
    ("fdtd_update_g", c_i32, [c_vp, _P(FdtdBuffers), c_vp]),
    ("fdtd_update_j", c_i32, [c_vp, _P(FdtdBuffers), c_vp, c_f64, c_f64, _P(c_i64)]),
    ("fdtd_monitor_sample", c_i32, [c_vp, _P(FdtdBuffers), c_vp, _P(FdtdDftMonitor)]),
    ("fdtd_plane_sum", c_i32, [c_vp, c_vp, c_i32, c_i32, c_i64, c_vp, c_i32, c_vp, c_vp]),
    ("fdtd_energy", c_i32, [c_vp, _P(FdtdBuffers), c_vp, c_i32, c_vp, c_vp]),
    ("fdtd_count_nonfinite", c_i32, [c_vp, _P(FdtdBuffers), c_vp, c_vp]),
    ("fdtd_plane_sum_noalloc", c_i32, [c_vp, c_vp, c_i32, c_i32, c_i64, c_i32, c_vp, c_vp]),
    ("fdtd_run", c_i32, [c_vp, _P(FdtdBuffers), c_vp, c_i32, _P(FdtdPointSources),
                         _P(FdtdDftMonitor)]),
    ("fdtd_run_kernel_ms", c_i32, [c_vp, _P(c_f64), _P(c_i32)]),
    ("fdtd_device_status", c_i32, [c_vp, c_vp, _P(c_i32)]),
    ("fdtd_batch_create", c_i32, [_P(FdtdBatchVariant), c_i32, c_i32, c_i64, _P(c_vp)]),
    ("fdtd_batch_destroy", c_i32, [c_vp]),
    ("fdtd_batch_tune", c_i32, [c_vp, c_i32, c_i32]),
    ("fdtd_batch_schedule", c_i32, [c_vp, c_i32]),
    ("fdtd_batch_run", c_i32, [c_vp, c_vp, c_i32]),
    ("fdtd_batch_get_step", c_i32, [c_vp, _P(c_i64)]),
    ("fdtd_batch_set_step", c_i32, [c_vp, c_i64]),
    ("fdtd_batch_encode", c_i32, [c_vp, c_i32, c_i32, c_vp, c_vp]),
    ("fdtd_batch_decode", c_i32, [c_vp, c_i32, c_i32, c_vp, c_vp]),
    ("fdtd_lbc_columns", c_i32, [_P(c_i32), c_i32, _P(c_i32), _P(c_i32)]),
    ("fdtd_lbc_gather", c_i32, [_P(c_i32), c_i32, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    ("fdtd_mlp_forward", c_i32, [c_vp, c_vp, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    ("fdtd_mlp_backward_workspace", c_i32, [c_i32, _P(c_i64)]),
    ("fdtd_mlp_backward", c_i32, [c_vp, c_vp, c_vp, c_vp, c_vp, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp,
                                  c_i64, c_vp]),
    ("fdtd_gram_workspace", c_i32, [c_i32, c_i32, c_i32, _P(c_i64)]),
    ("fdtd_gram", c_i32, [c_vp, c_i32, c_i32, c_vp, c_i32, c_vp, c_vp, c_i64, c_vp]),
    ("fdtd_adam", c_i32, [c_vp, c_vp, c_vp, c_vp, c_i32, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                          ctypes.c_float, c_i32, c_vp]),
    ("fdtd_lbc_pack", c_i32, [c_vp, c_vp, c_vp]),
    ("fdtd_lbc_predict", c_i32, [_P(c_i32), c_i32, c_i32, c_i32, ctypes.c_float, c_vp, c_vp, c_vp, c_vp, c_i64,
                                 c_vp]),
    ("fdtd_lbc_fix", c_i32, [_P(c_i32), c_i32, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp, c_f64, c_vp]),
    ("fdtd_lbc_attach", c_i32, [c_vp, c_i32, c_i32, ctypes.c_float, c_vp, c_vp, c_i64]),
]

FDTD_LBC_IN = 108
FDTD_LBC_HID = 64
FDTD_LBC_OUT = 6
FDTD_LBC_NPARAM = 11526
FDTD_LBC_PACK_WORDS = 6024
FDTD_LBC_FIX_E = 1
FDTD_LBC_FIX_H = 2
FDTD_LBC_F32 = 0
FDTD_LBC_BF16 = 1
FDTD_LBC_BF16X2 = 2
FDTD_LBC_LINEAR = 3

_LIB = None
_LOCK = threading.Lock()


def library_path() -> str:
    return _build.LIB


def load(auto_build: bool = True):
    """Load libfdtd_gb300.so (building it first when nvcc is available)."""
    global _LIB
    with _LOCK:
        if _LIB is not None:
            return _LIB
        path = _build.LIB
        if auto_build:
            try:
                _build.build()
            except RuntimeError as e:
                if not os.path.exists(path):
                    raise RuntimeError("libfdtd_gb300.so is not built and the build failed: %s" % e)
        if not os.path.exists(path):
            raise RuntimeError("libfdtd_gb300.so is not built (run opencl_fdtd_gb300.build.build())")
        lib = ctypes.CDLL(path)
        for name, res, args in SIGNATURES:
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if lib.fdtd_abi_version() != 1:
            raise RuntimeError("libfdtd_gb300.so ABI version mismatch")
        _LIB = lib
        return lib


class FdtdError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__("%s (status %d)" % (msg, code))
        self.code = code


def check(rc: int):
    if rc != FDTD_OK:
        msg = load().fdtd_last_error().decode(errors="replace")
        raise FdtdError(rc, msg)
