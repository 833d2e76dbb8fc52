"""ctypes binding of the C ABI in ``include/magreete_gb300.h``.

The library is built in-tree by ``magreete_gb300.build`` (``__graft_entry__.build()``
does this).  Nothing here falls back to another implementation: if the
library is missing or a call fails, an exception is raised.
"""
from __future__ import annotations

import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmagreete_gb300.so")

MGT_OK = 0
MGT_ERR_ARG = -1
MGT_ERR_CUDA = -2
MGT_ERR_SINGULAR = -3
MGT_ERR_TIMEOUT = -4
MGT_ERR_WORKSPACE = -5
MGT_ERR_UNSUPPORTED = -6
MGT_ERR_NOT_CONVERGED = -7

MGT_2D_VECTOR, MGT_2D_SCALAR, MGT_3D_VECTOR, MGT_3D_SCALAR = 0, 1, 2, 3
MGT_C128, MGT_C64, MGT_CDF = 0, 1, 2
MGT_NAN_KEEP, MGT_NAN_FILL = 0, 1
MGT_TUNE_PANEL_ROWS, MGT_TUNE_OUTER_BLOCK, MGT_TUNE_PANEL_MAX_CTAS, MGT_TUNE_COOPERATIVE = 1, 2, 3, 4
MGT_TUNE_PANEL_REGISTERS = 5
MGT_TUNE_TC_PRECISION = 6
MGT_TUNE_LOOKAHEAD = 7
MGT_TUNE_FUSED_RIGHT = 8
MGT_TUNE_PANEL_CLUSTER = 9
MGT_TUNE_SYM_ASSEMBLY = 10
MGT_TUNE_WIDE_UPDATE = 11
MGT_TC_TF32X3, MGT_TC_F16X2 = 0, 1
MGT_PIVOT_PARTIAL, MGT_PIVOT_TILE = 0, 1

class LuOptions(ctypes.Structure):
    """mgt_lu_options: per-call choices of one LU factorisation (zero / -1
    fields take the process-wide tuning values)."""
    _fields_ = [("size", ctypes.c_int32), ("pivoting", ctypes.c_int32), ("panel_rows", ctypes.c_int32),
                ("panel_max_ctas", ctypes.c_int32), ("cooperative", ctypes.c_int32), ("lookahead", ctypes.c_int32),
                ("outer_block", ctypes.c_int32)]

    def __init__(self, pivoting=0, panel_rows=0, panel_max_ctas=0, cooperative=-1, lookahead=-1, outer_block=0):
        super().__init__(ctypes.sizeof(LuOptions), pivoting, panel_rows, panel_max_ctas, cooperative, lookahead,
                         outer_block)


_vp = ctypes.c_void_p
_i64 = ctypes.c_int64
_i32 = ctypes.c_int
_f64 = ctypes.c_double
_sz = ctypes.c_size_t

# name -> (restype, argtypes); every symbol include/magreete_gb300.h declares
SIGNATURES = {
    "mgt_abi_version": (_i32, []),
    "mgt_status_string": (ctypes.c_char_p, [_i32]),
    "mgt_assemble_system": (_i32, [_i32, _vp, _i64, _f64, _f64, _f64, _f64, _f64, _vp, _i64, _i32, _vp, _i64, _i32, _vp]),
    "mgt_assemble_propagator": (_i32, [_i32, _vp, _i64, _vp, _i64, _f64, _f64, _f64, _i32, _f64, _i32, _f64, _f64,
                                       _i32, _vp, _i64, _vp]),
    "mgt_lu_workspace_bytes": (_i32, [_i32, _i64, ctypes.POINTER(_sz)]),
    "mgt_lu_factor": (_i32, [_i32, _vp, _i64, _i64, _vp, _vp, _sz, _vp]),
    "mgt_lu_factor_static": (_i32, [_i32, _vp, _i64, _i64, _vp, _vp, _vp]),
    "mgt_lu_factor_ex": (_i32, [_i32, _vp, _i64, _i64, _vp, _vp, _sz, ctypes.POINTER(LuOptions), _vp]),
    "mgt_lu_solve_workspace_bytes": (_i32, [_i32, _i64, _i64, ctypes.POINTER(_sz)]),
    "mgt_lu_solve": (_i32, [_i32, _vp, _i64, _i64, _vp, _vp, _i64, _vp, _i64, _i64, _vp, _sz, _vp]),
    "mgt_workspace_status": (_i32, [_vp, ctypes.POINTER(ctypes.c_int32), _vp]),
    "mgt_residual_workspace_bytes": (_i32, [_i64, _i64, ctypes.POINTER(_sz)]),
    "mgt_residual": (_i32, [_vp, _i64, _i64, _vp, _i64, _vp, _i64, _vp, _i64, _i64, _vp, _sz, _vp]),
    "mgt_residual_prepare": (_i32, [_vp, _i64, _i64, _vp, _sz, _vp]),
    "mgt_refine_prepare": (_i32, [_vp, _i64, _i64, _i64, _vp, _sz, _vp]),
    "mgt_residual_apply": (_i32, [_i64, _vp, _i64, _vp, _i64, _vp, _i64, _i64, _vp, _sz, _vp]),
    "mgt_refine_workspace_bytes": (_i32, [_i64, _i64, ctypes.POINTER(_sz)]),
    "mgt_solve_refined": (_i32, [_vp, _i64, _vp, _i64, _vp, _i64, _vp, _i64, _vp, _i64, _i64, _f64, _i32, _vp, _sz,
                                 ctypes.POINTER(_i32), ctypes.POINTER(_f64), _vp]),
    "mgt_refine_start": (_i32, [_vp, _i64, _vp, _i64, _vp, _i64, _vp, _i64, _i64, _vp, _sz, _vp]),
    "mgt_refine_correct": (_i32, [_vp, _i64, _vp, _i64, _vp, _i64, _vp, _i64, _vp, _i64, _i64, _vp, _sz, _vp]),
    "mgt_refine_norms": (_i32, [_vp, _i64, _i64, _vp, _i64, _vp, _i64, _i64, _vp, _sz, _vp, _vp]),
    "mgt_propagate_workspace_bytes": (_i32, [_i32, _i64, _i64, _i64, ctypes.POINTER(_sz)]),
    "mgt_propagate": (_i32, [_i32, _i32, _vp, _i64, _vp, _i64, _f64, _f64, _f64, _i32, _f64, _vp, _i64, _vp, _i64,
                             _vp, _i64, _i64, _vp, _sz, _vp]),
    "mgt_column_dots": (_i32, [_vp, _i64, _vp, _i64, _i64, _i64, _vp, _vp]),
    "mgt_cgemm_workspace_bytes": (_i32, [_i64, ctypes.POINTER(_sz)]),
    "mgt_cgemm_sub": (_i32, [_i32, _i32, _i64, _i64, _i64, _vp, _i64, _vp, _i64, _vp, _i64, _vp, _sz, _vp]),
    "mgt_set_tuning": (_i32, [_i32, _i32]),
    "mgt_get_tuning": (_i32, [_i32]),
    "mgt_diag_reset": (_i32, [_i32]),
    "mgt_diag_read": (_i32, [ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64),
                             ctypes.POINTER(_f64), ctypes.POINTER(_f64), ctypes.POINTER(_f64)]),
}

_lock = threading.Lock()
_lib = None


class MagreeteError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, status, where=""):
        self.status = status
        msg = _status_text(status)
        super().__init__(f"{where}: {msg} (status {status})" if where else f"{msg} (status {status})")


def _status_text(status):
    try:
        return load().mgt_status_string(status).decode()
    except Exception:  # library not loadable: still give a readable error
        return f"status {status}"


def load(path=None):
    """Load (once) and return the ctypes library handle."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise ImportError(
                f"{p} is missing: build the CUDA library first (python -c 'import __graft_entry__ as g; g.build()')")
        lib = ctypes.CDLL(p)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(status, where=""):
    if status != MGT_OK:
        raise MagreeteError(status, where)
    return status


def diag_reset(enable_timing=False):
    check(load().mgt_diag_reset(int(bool(enable_timing))), "mgt_diag_reset")


def diag_read():
    """(launches, dominant-kernel launches, ms, flops, bytes) since the last reset."""
    a, b = ctypes.c_uint64(), ctypes.c_uint64()
    ms, fl, by = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    check(load().mgt_diag_read(ctypes.byref(a), ctypes.byref(b), ctypes.byref(ms), ctypes.byref(fl),
                               ctypes.byref(by)), "mgt_diag_read")
    return a.value, b.value, ms.value, fl.value, by.value
