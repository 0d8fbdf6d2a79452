"""ctypes binding of libmtgpu (include/mtgpu.h).

The library is loaded from the package's in-tree _build/ directory.  There
is no fallback: if the shared object is missing or fails to load, every call
raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_build", "libmtgpu.so")

_i = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_d = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_vp = C.c_void_p

MTGPU_OK = 0
MTGPU_X0_NULL = -1
MTGPU_DIV_BY_ZERO = -2
MTGPU_MAXITER = -3
MTGPU_ERR_ARG = -101
MTGPU_ERR_CUDA = -102
MTGPU_ERR_IO = -103
MTGPU_ERR_UNSUPPORTED = -104
MTGPU_ERR_TIMEOUT = -105
MTGPU_NOALLOC_NOT_ZERO_BASED = 1
MTGPU_NOALLOC_BAD_ENTRY = 2


class SolveStats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("residual_rel", C.c_double),
                ("true_residual_rel", C.c_double), ("setup_seconds", C.c_double),
                ("solve_seconds", C.c_double), ("status", C.c_int), ("spmv_variant", C.c_int),
                ("matfree_check", C.c_double)]


class SolveOpts(C.Structure):
    _fields_ = [("stop_on_true_residual", C.c_int), ("iterations_per_launch", C.c_int),
                ("double_float", C.c_int)]


class FemMesh(C.Structure):
    _fields_ = [("kuzlov", C.c_int), ("kpar", C.c_int), ("nb", C.c_int), ("n_materials", C.c_int),
                ("xyz", C.c_void_p), ("nver", C.c_void_p), ("nver_stride", C.c_int),
                ("ed", C.c_void_p), ("ed_stride", C.c_int), ("edges", C.c_void_p),
                ("nvkat", C.c_void_p), ("mu", C.c_void_p), ("mu0", C.c_void_p),
                ("sigma", C.c_void_p), ("sigma0", C.c_void_p), ("dpr", C.c_void_p),
                ("dpr0", C.c_void_p), ("n_bound", C.c_int), ("bound_nodes", C.c_void_p)]


SURVEY_MAX_SYSTEMS = 256   # MTGPU_SURVEY_MAX_SYSTEMS


class SurveyStats(C.Structure):
    _fields_ = [("status", C.c_int * SURVEY_MAX_SYSTEMS),
                ("iterations", C.c_int * SURVEY_MAX_SYSTEMS),
                ("verifications", C.c_int * SURVEY_MAX_SYSTEMS),
                ("fp64_iterations", C.c_int * SURVEY_MAX_SYSTEMS),
                ("true_residual_rel", C.c_double * SURVEY_MAX_SYSTEMS),
                ("residual_rel", C.c_double * SURVEY_MAX_SYSTEMS),
                ("seconds", C.c_double)]


class MtgpuError(RuntimeError):
    pass


# (name, restype, argtypes) of every exported entry point
SIGNATURES = {
    "mtgpu_last_error": (C.c_char_p, []),
    "mtgpu_kernel_launches": (C.c_ulonglong, []),
    "mtgpu_pcocr_2x2_folded": (C.c_int, [
        C.c_int, _i, _i, _i, _i, _d, _d, _d, _d, C.c_double, C.c_int, _vp,
        C.c_int, C.c_int, C.c_int, _d, _i, _i, _d, _i, _i, _i, _d, _i]),
    "mtgpu_pcocr_2x2_folded_ex": (C.c_int, [
        C.c_int, _i, _i, _i, _i, _d, _d, _d, _d, C.c_double, C.c_int,
        C.c_int, C.c_int, C.c_int, _d, _i, _i, _d, _i, _i, _i, _d, _i,
        C.POINTER(SolveOpts), C.POINTER(SolveStats)]),
    "mtgpu_mult_mv_block_2x2": (C.c_int, [C.c_int, _i, _i, _i, _i, _d, _d, _d, _d]),
    "mtgpu_mult_mv_block_2x2_noalloc": (C.c_int, [C.c_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                                  _vp, _vp, _vp]),
    "mtgpu_folded_apply": (C.c_int, [
        C.c_int, _i, _i, _i, _i, _d, _d, C.c_int, C.c_int, _i, _i, _d, _i, _i, _i, _d, _i,
        _d, _d, C.POINTER(C.c_int), _vp, _vp]),
    "mtgpu_cocr_create": (C.c_int, [
        C.c_int, C.c_int, _vp, _vp, _vp, _vp, _vp, _vp, C.c_int,
        C.c_int, C.c_int, _i, _i, _d, _i, _i, _i, _d, _i, _vp, C.POINTER(_vp)]),
    "mtgpu_cocr_solve": (C.c_int, [_vp, _vp, _vp, C.c_double, C.c_int,
                                   C.POINTER(SolveOpts), C.POINTER(SolveStats)]),
    "mtgpu_cocr_spmv": (C.c_int, [_vp, _vp, _vp]),
    "mtgpu_cocr_spmv_timed": (C.c_int, [_vp, _vp, _vp, C.c_int, C.POINTER(C.c_float)]),
    "mtgpu_cocr_precond": (C.c_int, [_vp, _vp, _vp]),
    "mtgpu_cocr_info": (C.c_int, [_vp, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong),
                                  C.POINTER(C.c_int)]),
    "mtgpu_cocr_destroy": (None, [_vp]),
    "mtgpu_assembly_create_regular": (C.c_int, [C.c_int, C.c_int, C.c_int, _d, _d, _d, _i, C.c_int,
                                                _d, _d, _d, C.POINTER(_vp)]),
    "mtgpu_assembly_create": (C.c_int, [C.POINTER(FemMesh), C.POINTER(_vp)]),
    "mtgpu_assembly_info": (C.c_int, [_vp, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong),
                                      C.POINTER(C.c_int), C.POINTER(C.c_longlong)]),
    "mtgpu_assembly_block2x2": (C.c_int, [_vp, C.c_double, C.c_int, C.c_int, _d, _d, _d,
                                          _i, _i, _i, _i, _d, _d, _d]),
    "mtgpu_assembly_rhs": (C.c_int, [_vp, C.c_int, _d, _i, C.c_int, _d, _d, _d, _vp]),
    "mtgpu_cocr_create_from_assembly": (C.c_int, [_vp, C.c_double, _vp, C.POINTER(_vp)]),
    "mtgpu_assembly_check_preconditioner": (C.c_int, [_vp, C.POINTER(C.c_int)]),
    "mtgpu_assembly_destroy": (None, [_vp]),
    "mtgpu_survey_create": (C.c_int, [_vp, C.c_int, _d, _vp, C.POINTER(_vp)]),
    "mtgpu_survey_solve": (C.c_int, [_vp, _vp, _vp, C.c_double, C.c_int, C.c_int,
                                     C.POINTER(SurveyStats)]),
    "mtgpu_survey_create_multi": (C.c_int, [C.c_int, C.POINTER(_vp), _i, _d, _vp, C.POINTER(_vp)]),
    "mtgpu_survey_info": (C.c_int, [_vp, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                    C.POINTER(C.c_longlong)]),
    "mtgpu_survey_preconditioner": (C.c_int, [_vp, C.POINTER(C.c_int), C.POINTER(C.c_float)]),
    "mtgpu_survey_spmv": (C.c_int, [_vp, _vp, _vp]),
    "mtgpu_survey_spmv_timed": (C.c_int, [_vp, C.c_int, C.POINTER(C.c_float)]),
    "mtgpu_survey_tuning": (C.c_int, [_vp, C.POINTER(C.c_int), C.POINTER(C.c_float)]),
    "mtgpu_survey_set_spmv_variant": (C.c_int, [_vp, C.c_int]),
    "mtgpu_survey_destroy": (None, [_vp]),
    "mtgpu_receivers_create": (C.c_int, [_vp, C.c_int, _d, C.POINTER(_vp)]),
    "mtgpu_receivers_info": (C.c_int, [_vp, C.POINTER(C.c_int), C.POINTER(C.c_int), _vp]),
    "mtgpu_receivers_fields": (C.c_int, [_vp, C.c_int, _d, _i, C.c_int, _d, _d, _d, _vp, _vp,
                                         _vp, _vp]),
    "mtgpu_mt_response": (C.c_int, [_vp, C.c_int, _d, _i, _i, C.c_int, _vp, _vp, _vp]),
    "mtgpu_receivers_destroy": (None, [_vp]),
    "mtgpu_receivers_set_output": (C.c_int, [_vp, _vp, C.c_int, C.c_int]),
    "mtgpu_receivers_smoothing_info": (C.c_int, [_vp, C.c_int, C.POINTER(C.c_int), _vp, _vp,
                                                 _vp, C.POINTER(C.c_int)]),
    "mtgpu_adjoint_source": (C.c_int, [_vp, C.c_int, _d, _i, _i, C.c_int, _vp, _vp, _vp, _vp,
                                       C.POINTER(C.c_double)]),
    "mtgpu_adjoint_gradient": (C.c_int, [_vp, C.c_int, _d, _i, C.c_int, _d, _d, _d, _vp, _vp,
                                         _vp]),
}

_lib = None


def lib():
    """Load libmtgpu; raises if it is not built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise MtgpuError(f"libmtgpu is not built ({LIB_PATH} missing); "
                             "run __graft_entry__.build() or python -m "
                             "mtcalc_with_dfp_cocr_gb300.build")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def last_error() -> str:
    s = lib().mtgpu_last_error()
    return s.decode() if s else ""


def check(rc: int, what: str) -> int:
    """Raise on library errors (codes below -100); solver codes pass through."""
    if rc <= -100:
        raise MtgpuError(f"{what} failed ({rc}): {last_error()}")
    return rc


def kernel_launches() -> int:
    return int(lib().mtgpu_kernel_launches())
