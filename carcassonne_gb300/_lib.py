"""ctypes binding of libcarcgb300.so, the C ABI declared in include/carcassonne_gb300.h.

The library is built in-tree (``carcassonne_gb300/build.py``).  Loading it is
mandatory for every compute call: there is no CPU or library fallback, and a
missing library raises ``RuntimeError`` at the first call.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

CARC_HEGV_TENSOR_CORE = 1
CARC_HEGV_SINGLE = 2
CARC_OK = 0
CARC_BAD_SHAPE = 1
CARC_BAD_ARG = 2
CARC_CUDA_ERROR = 3
CARC_NOT_CONVERGED = 4
CARC_NAN = 5
CARC_NOT_POSDEF = 6
CARC_TOO_LARGE = 7
CARC_RELAX_FAILED = 8

MAX_SUBDIMS = 6
MAX_SLOTS = 64
MAX_ENTRIES = 512

_i32, _i64, _dbl, _vp = ctypes.c_int32, ctypes.c_int64, ctypes.c_double, ctypes.c_void_p
_pvp = ctypes.POINTER(ctypes.c_void_p)
_pi32 = ctypes.POINTER(ctypes.c_int32)
_pi64 = ctypes.POINTER(ctypes.c_int64)


class ContractDesc(ctypes.Structure):
    _fields_ = [
        ("nm", _i32), ("nn", _i32), ("nk", _i32), ("conj_a", _i32), ("conj_b", _i32),
        ("m_ext", _i64 * MAX_SUBDIMS), ("n_ext", _i64 * MAX_SUBDIMS), ("k_ext", _i64 * MAX_SUBDIMS),
        ("a_m", _i64 * MAX_SUBDIMS), ("a_k", _i64 * MAX_SUBDIMS),
        ("b_n", _i64 * MAX_SUBDIMS), ("b_k", _i64 * MAX_SUBDIMS),
        ("c_m", _i64 * MAX_SUBDIMS), ("c_n", _i64 * MAX_SUBDIMS),
    ]


# name -> (restype, argtypes)
SIGNATURES = {
    "carc_last_error_string": (ctypes.c_char_p, []),
    "carc_version": (ctypes.c_int, []),
    "carc_launch_counter": (_i64, []),
    "carc_phase_timing_enable": (_i32, [_i32]),
    "carc_host_alloc_mapped": (ctypes.c_int, [_i64, ctypes.POINTER(_vp), ctypes.POINTER(_vp)]),
    "carc_host_free": (ctypes.c_int, [_vp]),
    "carc_phase_timing_read": (_i32, [_i32, ctypes.POINTER(ctypes.c_double), _pi64]),
    "carc_zcontract_grouped": (ctypes.c_int, [ctypes.POINTER(ContractDesc), _pvp, _i32, _pvp, _i32, _pvp, _i32,
                                              _pi32, _i32, _dbl, _dbl, _i32, _vp, _i64, _vp]),
    "carc_zcontract_workspace_size": (_i64, [ctypes.POINTER(ContractDesc), _i32]),
    "carc_zpermute": (ctypes.c_int, [_vp, _vp, _i32, _pi64, _pi64, _i32, _vp]),
    "carc_zaxpby": (ctypes.c_int, [_i64, _dbl, _dbl, _vp, _dbl, _dbl, _vp, _vp, _vp]),
    "carc_zmul": (ctypes.c_int, [_i64, _vp, _vp, _vp, _vp]),
    "carc_zfill": (ctypes.c_int, [_i64, _dbl, _dbl, _vp, _vp]),
    "carc_zdot": (ctypes.c_int, [_i64, _vp, _vp, _i32, _vp, _vp, _i64, _vp]),
    "carc_zdot_workspace_size": (_i64, [_i64]),
    "carc_zhasnan": (ctypes.c_int, [_i64, _vp, _vp, _vp]),
    "carc_stage3_matvec_f64": (ctypes.c_int, [_pi64, _pi64, _i64, _pvp, _i32, _pvp, _i32, _pvp, _i32, _pi32, _i32,
                                              _vp, _vp, _i32, _i32, _vp, _i64, _vp]),
    "carc_stage3_matvec_f64_workspace_size": (_i64, [_pi64, _pi64, _i64, _i32, _i32]),
    "carc_stage3_matvec_f64_noalloc": (ctypes.c_int, [_pi64, _pi64, _i64, _pvp, _i32, _pvp, _i32, _pvp, _i32, _pi32,
                                                      _i32, _vp, _vp, _i32, _i32, _vp]),
    "carc_stage3_form_matrix_f64": (ctypes.c_int, [_pi64, _pi64, _i64, _pvp, _i32, _pvp, _i32, _pvp, _i32, _pi32,
                                                   _i32, _vp, _i32, _vp, _i64, _vp]),
    "carc_stage3_form_matrix_f64_workspace_size": (_i64, [_pi64, _pi64, _i64, _i32]),
    "carc_zgesvd_jacobi": (ctypes.c_int, [_i32, _i32, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _i64, _vp]),
    "carc_zgesvd_jacobi_workspace_size": (_i64, [_i32, _i32, _i32]),
    "carc_normalize_axis_finish": (ctypes.c_int, [_i32, _vp, _vp, _dbl, _i32, _vp, _vp, _vp]),
    "carc_zgeqr_economic": (ctypes.c_int, [_i32, _i32, _vp, _vp, _vp, _vp]),
    "carc_zheev_jacobi": (ctypes.c_int, [_i32, _i32, _vp, _vp, _vp, _vp, _vp, _i64, _vp]),
    "carc_zheev_jacobi_workspace_size": (_i64, [_i32, _i32]),
    "carc_zpotrf": (ctypes.c_int, [_i32, _vp, _vp, _vp, _i64, _vp]),
    "carc_zpotrf_workspace_size": (_i64, [_i32]),
    "carc_ztrtri_lower": (ctypes.c_int, [_i32, _vp, _vp, _vp, _i64, _vp]),
    "carc_ztrtri_lower_workspace_size": (_i64, [_i32]),
    "carc_zhegv_lowest": (ctypes.c_int, [_i32, _vp, _vp, _vp, _vp, ctypes.POINTER(_dbl), _i32, _i32, _dbl, _i32,
                                         ctypes.POINTER(_i32), _vp, _vp, _i64, _vp]),
    "carc_zhegv_lowest_workspace_size": (_i64, [_i32, _i32, _i32]),
    "carc_zheev_lowest_lanczos": (ctypes.c_int, [_i32, _vp, _vp, _vp, ctypes.POINTER(_dbl), _i32, _i32, _dbl,
                                                 ctypes.POINTER(_i32), _vp, _i64, _vp]),
    "carc_zheev_lowest_lanczos_workspace_size": (_i64, [_i32, _i32]),
    "carc_zminres_projected": (ctypes.c_int, [_i32, _vp, _vp, _dbl, _vp, _vp, _i32, _dbl, ctypes.POINTER(_i32), _vp,
                                              _i64, _vp]),
    "carc_zminres_projected_workspace_size": (_i64, [_i32]),
    "carc_zcg_hpsd": (ctypes.c_int, [_i32, _vp, _vp, _vp, _dbl, _i32, _vp, _vp, _vp]),
    "carc_zcg_hpsd_grid": (ctypes.c_int, [_i32, _vp, _vp, _vp, _dbl, _i32, _vp, _vp, _vp, _i64, _vp]),
    "carc_zcg_hpsd_grid_workspace_size": (_i64, [_i32]),
    "carc_mlp_linear_forward": (ctypes.c_int, [_i32, _i32, _i32, _vp, _vp, _vp, _i32, _vp, _vp]),
    "carc_mlp_linear_backward": (ctypes.c_int, [_i32, _i32, _i32, _vp, _vp, _vp, _vp, _i32, _vp, _vp, _vp, _vp, _vp]),
    "carc_mlp_mse": (ctypes.c_int, [_i64, _i32, _vp, _vp, _vp, _vp, _vp]),
    "carc_mlp_adam": (ctypes.c_int, [_i64, _vp, _vp, _vp, _vp, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                     ctypes.c_float, _i32, _vp]),
    "carc_mlp_to_bf16": (ctypes.c_int, [_i64, _vp, _vp, _vp]),
    "carc_mlp_linear_bf16": (ctypes.c_int, [_i32, _i32, _i32, _vp, _vp, _vp, _i32, _vp, _vp, _vp]),
    "carc_relax_over": (ctypes.c_int, [_i32, _vp, _vp, _vp, _vp, _i32, _i32, _dbl, ctypes.POINTER(_dbl),
                                       ctypes.POINTER(_i32), ctypes.POINTER(_dbl), _vp, _i64, _vp]),
    "carc_relax_over_workspace_size": (_i64, [_i32, _i32]),
    "carc_lobpcg_workspace_size": (_i64, [_i32, _i32]),
    "carc_lobpcg_inner": (ctypes.c_int, [_i32, _i32, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i32, _i32, _vp, _vp,
                                         _i32, _i32, _vp, _vp, _vp, _i64, _vp]),
    "carc_lobpcg_orth_prepare": (ctypes.c_int, [_i32, _i32, _vp, _vp, _dbl, _vp, _vp, _vp]),
    "carc_lobpcg_orth_finish": (ctypes.c_int, [_i32, _i32, _vp, _vp, _vp, _vp, _vp, _dbl, _i32, _vp, _vp]),
    "carc_lobpcg_orth_apply": (ctypes.c_int, [_i32, _i32, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                              _vp]),
    "carc_lobpcg_rr_scale": (ctypes.c_int, [_i32, _i32, _vp, _vp, _vp, _vp, _vp]),
    "carc_lobpcg_rr_reduce": (ctypes.c_int, [_i32, _i32, _vp, _vp, _vp, _vp, _vp, _dbl, _vp, _vp, _vp, _vp]),
    "carc_lobpcg_rr_combine": (ctypes.c_int, [_i32, _i32, _vp, _vp, _vp, _vp, _vp]),
    "carc_lobpcg_update": (ctypes.c_int, [_i32, _i32, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                          _vp, _vp, _vp, _vp, _vp, _i64, _vp]),
    "carc_zcontract_tc": (ctypes.c_int, [ctypes.POINTER(ContractDesc), _vp, _vp, _vp, _dbl, _dbl, _i32, _i32, _vp, _i64,
                                         _vp, _vp]),
    "carc_zcontract_tc_workspace_size": (_i64, [ctypes.POINTER(ContractDesc), _i32]),
    "carc_zcontract_tc_grouped": (ctypes.c_int, [ctypes.POINTER(ContractDesc), _pvp, _i32, _pvp, _i32, _pvp, _i32,
                                                 _pi32, _i32, _dbl, _dbl, _i32, _vp, _i64, _vp, _vp]),
    "carc_zcontract_tc_grouped_workspace_size": (_i64, [ctypes.POINTER(ContractDesc), _i32, _i32, _i32]),
    "carc_stage3_tc_plan_size": (_i64, [_pi64, _pi64, _pi32, _i32]),
    "carc_stage3_tc_prepare": (ctypes.c_int, [_pi64, _pi64, _pvp, _i32, _pvp, _i32, _pi32, _i32, _vp, _i64, _vp]),
    "carc_stage3_matvec_tc": (ctypes.c_int, [_pi64, _pi64, _i64, _vp, _i32, _i32, _pvp, _i32, _pi32, _i32, _vp, _vp,
                                             _i32, _i32, _vp, _i64, _vp, _vp]),
    "carc_stage3_matvec_tc_workspace_size": (_i64, [_pi64, _pi64, _i64, _pi32, _i32, _i32]),
    "carc_tc_autotune_set": (ctypes.c_int, [_pi64, _pi64, _i64, _i32, _i32, _i32]),
    "carc_tc_autotune_clear": (ctypes.c_int, []),
    "carc_tc_autotune_set_fold": (ctypes.c_int, [_pi64, _pi64, _i64, _i32, _i32, _i32]),
    "carc_stage3_form_matrix_tc": (ctypes.c_int, [_pi64, _pi64, _i64, _pvp, _i32, _pvp, _i32, _pvp, _i32, _pi32, _i32,
                                                  _vp, _i32, _vp, _i64, _vp, _vp]),
    "carc_stage3_form_matrix_tc_workspace_size": (_i64, [_pi64, _pi64, _i64, _i32]),
    "carc_gemm_bf16_tn": (ctypes.c_int, [_vp, _i32, _vp, _i32, _i32, _vp, _i64, _i32, _vp, _vp]),
}

_lock = threading.Lock()
_lib = None


class CarcError(RuntimeError):
    def __init__(self, status, message):
        RuntimeError.__init__(self, "carc status %d: %s" % (status, message))
        self.status = status


class CarcShapeError(CarcError, ValueError):
    pass


class CarcArgError(CarcError, ValueError):
    pass


class CarcNotConverged(CarcError):
    pass


def library_path():
    return _build.lib_path()


def load():
    """Load (and bind) the CUDA library; raise if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = library_path()
        if not os.path.exists(path):
            raise RuntimeError("libcarcgb300.so is not built (expected at %s); run "
                               "`python -m carcassonne_gb300.build`" % path)
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(status):
    if status == CARC_OK:
        return
    msg = load().carc_last_error_string().decode(errors="replace")
    if status == CARC_BAD_SHAPE:
        raise CarcShapeError(status, msg)
    if status in (CARC_BAD_ARG, CARC_TOO_LARGE):
        raise CarcArgError(status, msg)
    if status == CARC_NOT_CONVERGED:
        raise CarcNotConverged(status, msg)
    raise CarcError(status, msg)


def call(name, *args):
    check(getattr(load(), name)(*args))


def ptr_array(ptrs):
    arr = (ctypes.c_void_p * max(1, len(ptrs)))(*[ctypes.c_void_p(int(p)) for p in ptrs])
    return ctypes.cast(arr, _pvp), arr


def i32_array(vals):
    arr = (ctypes.c_int32 * max(1, len(vals)))(*[int(v) for v in vals])
    return ctypes.cast(arr, _pi32), arr


def i64_array(vals):
    arr = (ctypes.c_int64 * max(1, len(vals)))(*[int(v) for v in vals])
    return ctypes.cast(arr, _pi64), arr
