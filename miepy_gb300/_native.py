"""ctypes binding of the C ABI in ``include/miepy_gb300.h``.

The CUDA extension is the only compute path: if the shared library is missing
or no CUDA device is present, every call raises instead of falling back to the
CPU.
"""

from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

_lib = None
_lock = threading.Lock()

c_int, c_double, c_size_t, c_void_p, c_int64 = ctypes.c_int, ctypes.c_double, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_int64
_P = c_void_p

GB_OK, GB_NOT_CONVERGED, GB_BREAKDOWN, GB_NAN, GB_OVER_BUDGET, GB_TIMEOUT, GB_BAD_ARG, GB_CUDA_ERROR, GB_UNSUPPORTED = range(9)
PREC_FP64, PREC_MIXED, PREC_FP32, PREC_MIXED_FP64RES = 0, 1, 2, 3
STATUS_NAMES = {0: "ok", 1: "not converged", 2: "breakdown", 3: "nan", 4: "over budget", 5: "timeout",
                6: "bad argument", 7: "cuda error", 8: "unsupported", -1: "running"}


class GBError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"miepy_gb300 error {code} ({STATUS_NAMES.get(code, '?')}): {msg}")
        self.code = code


class gb_system(ctypes.Structure):
    _fields_ = [("N", ctypes.c_int32), ("lmax", ctypes.c_int32), ("k", c_double), ("pos_off", c_int64),
                ("mat_off", c_int64), ("vec_off", c_int64), ("t_off", c_int64)]


SIGNATURES = {
    "gb_version": (c_int, []),
    "gb_last_error": (c_size_t, [ctypes.c_char_p, c_size_t]),
    "gb_device_sm_count": (c_int, []),
    "gb_launch_count": (ctypes.c_longlong, []),
    "gb_tables_prepare": (c_int, [c_int, _P]),
    "gb_tables_count": (c_int, [c_int, ctypes.POINTER(c_int)]),
    "gb_tables_export": (c_int, [c_int, _P, _P, _P, _P, _P]),
    "gb_assemble_sphere_dense": (c_int, [c_int, c_int, _P, _P, c_double, _P, _P]),
    "gb_reflection_matrix_dense": (c_int, [c_int, c_int, _P, _P, c_double, c_double, c_double, c_double, _P, _P]),
    "gb_aggregate_periodic_dense": (c_int, [c_int, c_int, _P, _P, c_double, _P, c_int, c_double, c_double, c_double, _P,
                                            _P]),
    "gb_assemble_sphere_packed": (c_int, [c_int, c_int, _P, c_double, _P, _P, _P, _P]),
    "gb_assemble_batch": (c_int, [c_int, _P, _P, _P, _P, _P, _P]),
    "gb_expand_mie_batch": (c_int, [c_int, _P, _P, _P, _P, _P]),
    "gb_solve_workspace_size": (c_size_t, [c_int, _P, c_int, c_int]),
    "gb_solve_batch": (c_int, [c_int, _P, c_int, c_int, c_double, c_int, c_double, c_int, _P, _P, _P, _P, _P, _P,
                               _P, c_size_t, _P, _P, _P, _P]),
    "gb_solve_batch_ex": (c_int, [c_int, _P, c_int, c_int, c_double, c_int, c_double, c_int, _P, _P, _P, _P, _P, _P,
                                  _P, _P, _P, c_size_t, _P, _P, _P, _P]),
    "gb_sphere_preconditioner": (c_int, [ctypes.c_longlong, _P, _P, _P]),
    "gb_dense_precondition_matrix": (c_int, [c_int, c_int, _P, _P, _P, _P]),
    "gb_block_diag_apply": (c_int, [c_int, c_int, c_int, _P, _P, _P, _P]),
    "gb_tc_matrix_bytes": (c_size_t, [c_int, _P]),
    "gb_tc_matrix_build": (c_int, [c_int, _P, _P, _P, _P]),
    "gb_apply_repeat_tc": (c_int, [c_int, _P, c_int, _P, _P, _P, _P, _P, c_size_t, c_int, c_int, _P]),
    "gb_solve_dense_workspace_size": (c_size_t, [c_int, c_int]),
    "gb_solve_dense": (c_int, [c_int, c_int, _P, _P, _P, c_double, c_int, _P, c_size_t, _P, _P, _P, _P]),
    "gb_beam_project": (c_int, [c_int, c_int, c_int, _P, _P, _P, c_double, _P, c_int, _P]),
    "gb_cluster_coefficients_workspace_size": (c_size_t, [c_int, c_int]),
    "gb_cluster_coefficients": (c_int, [c_int, c_int, _P, _P, c_double, _P, c_int, _P, _P, c_size_t, _P]),
    "gb_far_field": (c_int, [c_int, c_int, _P, _P, c_double, _P, c_int, _P, _P, _P, c_int, c_double, c_double, _P,
                             _P]),
    "gb_solve_dense_noalloc": (c_int, [c_int, c_int, _P, _P, _P, c_double, c_int, _P, _P, _P, _P]),
    "gb_apply_workspace_size": (c_size_t, [c_int, _P, c_int, c_int]),
    "gb_apply_batch": (c_int, [c_int, _P, c_int, c_int, _P, _P, _P, _P, _P, _P, _P, c_size_t, _P]),
    "gb_apply_repeat": (c_int, [c_int, _P, c_int, c_int, _P, _P, _P, _P, _P, _P, _P, c_size_t, c_int, c_int, _P]),
    "gb_autotune_gemv": (c_int, [c_int, _P, c_int, c_int, _P, _P, _P, _P, _P, _P, c_size_t, c_int, _P]),
    "gb_gemv_shape": (c_int, [c_int, c_int, c_int, _P, _P]),
    "gb_set_gemv_wait_limit": (c_int, [ctypes.c_longlong, _P]),
    "gb_epilogue_batch": (c_int, [c_int, _P, c_int, _P, _P, _P, _P, _P, _P, c_double, c_int, _P, _P, _P, _P, _P,
                                  _P]),
    "gb_solve_batch_tmatrix": (c_int, [c_int, _P, c_int, c_int, c_double, c_int, c_double, c_int, _P, _P, _P, _P, _P,
                                       _P, _P, _P, _P, c_size_t, _P, _P, _P, _P]),
    "gb_tmatrix_epilogue_batch": (c_int, [c_int, _P, c_int, _P, _P, _P, _P, _P, c_double, c_int, _P, _P, _P, _P,
                                          _P]),
    "gb_particle_cross_sections": (c_int, [c_int, c_int, _P, _P, _P, c_double, _P, _P]),
    "gb_particle_aggregate_workspace_size": (c_size_t, [c_int, c_int]),
    "gb_particle_aggregate_dense": (c_int, [c_int, c_int, _P, _P, c_double, _P, c_size_t, _P, _P]),
    "gb_near_field": (c_int, [c_int, c_int, _P, _P, _P, _P, c_double, _P, c_int, _P, c_int, c_int, c_double, c_double,
                              _P, _P, _P]),
    "gb_near_field32": (c_int, [c_int, c_int, _P, _P, _P, _P, c_double, _P, c_int, _P, c_int, c_int, c_double,
                                c_double, _P, _P, _P]),
    "gb_far_field_expansions": (c_int, [c_int, c_int, _P, _P, c_double, c_int, _P, c_int, c_double, c_double, _P,
                                        _P]),
}


def lib_path() -> str:
    return _build.LIB


def lib():
    """Load (building first if needed) the CUDA extension."""
    global _lib
    with _lock:
        if _lib is None:
            path = _build.LIB
            if not _build.up_to_date():
                try:
                    _build.build()
                except Exception as e:   # no silent fallback: the extension is the product
                    raise RuntimeError(f"miepy_gb300 CUDA extension unavailable: {e}") from e
            L = ctypes.CDLL(path)
            for name, (res, args) in SIGNATURES.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            _lib = L
    return _lib


def last_error() -> str:
    buf = ctypes.create_string_buffer(1024)
    lib().gb_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def check(code: int, what: str = "") -> int:
    if code != GB_OK:
        raise GBError(code, (what + ": " if what else "") + last_error())
    return code


def ptr(t) -> int | None:
    """Raw device/host address of a torch tensor or numpy array (None passes NULL)."""
    if t is None:
        return None
    if hasattr(t, "data_ptr"):
        return t.data_ptr()
    return t.ctypes.data


def systems_array(descs):
    arr = (gb_system * len(descs))()
    for i, d in enumerate(descs):
        arr[i] = gb_system(*d)
    return arr
