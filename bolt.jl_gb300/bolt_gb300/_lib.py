"""ctypes binding of libbolt_gb300.so (include/bolt_gb300.h).

Loading fails loudly: there is no CPU fallback for the solver or the
line-of-sight kernels.  Only ``bolt_host_tables`` and the unit helpers work
without a GPU.
"""
from __future__ import annotations

import ctypes as C
import os

from . import _build

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_i32p = C.POINTER(C.c_int32)
_i64p = C.POINTER(C.c_int64)


class BoltParams(C.Structure):
    _fields_ = [(n, C.c_double) for n in
                ("h", "Omega_r", "Omega_b", "Omega_c", "A", "n", "Y_p", "N_nu", "Sigma_m_nu")]


class BoltGrid(C.Structure):
    _fields_ = [("start", C.c_double), ("step", C.c_double), ("stop", C.c_double)]


class BoltRecfast(C.Structure):
    _fields_ = [("Yp", C.c_double), ("OmegaB", C.c_double), ("OmegaG", C.c_double), ("Tnow", C.c_double),
                ("tol", C.c_double), ("ionization", C.c_int)]


class BoltHier(C.Structure):
    _fields_ = [("lg", C.c_int), ("lnu", C.c_int), ("lmnu", C.c_int), ("nq", C.c_int)]


class BoltOpts(C.Structure):
    _fields_ = [("device", C.c_int), ("warps_per_block", C.c_int), ("max_steps", C.c_longlong)]


class BoltRequest(C.Structure):
    _fields_ = [("kind", C.c_int), ("grad", C.c_int), ("par", BoltParams), ("grid", BoltGrid), ("nq", C.c_int),
                ("hier", BoltHier), ("reltol", C.c_double), ("abstol", C.c_double), ("k", _dp), ("nk", C.c_int),
                ("plin_x", C.c_double), ("ells", _ip), ("nell", C.c_int), ("cl_want", C.c_int),
                ("plin", _dp), ("dplin", _dp), ("tt", _dp), ("te", _dp), ("ee", _dp), ("dtt", _dp), ("dte", _dp),
                ("dee", _dp), ("status", _i32p)]


class BoltEngineCfg(C.Structure):
    _fields_ = [("device", C.c_int), ("lanes", C.c_int), ("host_threads", C.c_int), ("max_batch", C.c_int),
                ("mem_budget_gb", C.c_double), ("warps_per_mode", C.c_int), ("max_steps", C.c_longlong),
                ("batch_window_s", C.c_double), ("objective", C.c_int),
                ("land_stride", C.c_int), ("grad_scheme", C.c_int)]


EXPORTS = {
    "bolt_version": (C.c_int, []),
    "bolt_mass_natural": (C.c_double, []),
    "bolt_km_s_Mpc_100": (C.c_double, []),
    "bolt_host_tables": (C.c_int, [C.POINTER(BoltParams), C.POINTER(BoltGrid), C.c_int, C.POINTER(BoltRecfast),
                                   _dp, _dp, C.c_char_p, C.c_int]),
    "bolt_host_tables_frozen": (C.c_int, [C.POINTER(BoltParams), C.POINTER(BoltParams), C.POINTER(BoltGrid), C.c_int,
                                          C.POINTER(BoltRecfast), C.POINTER(BoltRecfast), _dp, C.c_char_p, C.c_int]),
    "bolt_ctx_create": (C.c_int, [C.POINTER(BoltOpts), C.POINTER(C.c_void_p)]),
    "bolt_ctx_destroy": (None, [C.c_void_p]),
    "bolt_last_error": (C.c_char_p, [C.c_void_p]),
    "bolt_cosmo_build": (C.c_int, [C.c_void_p, C.POINTER(BoltParams), C.POINTER(BoltGrid), C.c_int,
                                   C.POINTER(BoltRecfast), _ip]),
    "bolt_cosmo_upload": (C.c_int, [C.c_void_p, C.POINTER(BoltParams), C.POINTER(BoltGrid), C.c_int, _dp, _dp,
                                    _ip]),
    "bolt_cosmo_info": (C.c_int, [C.c_void_p, C.c_int, _dp]),
    "bolt_cosmo_table": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _dp]),
    "bolt_cosmo_free": (C.c_int, [C.c_void_p, C.c_int]),
    "bolt_boltsolve": (C.c_int, [C.c_void_p, C.c_int, _dp, C.c_int, C.POINTER(BoltHier), C.c_double, C.c_double,
                                 _dp, C.c_int, _dp, _i32p]),
    "bolt_boltsolve_rsa": (C.c_int, [C.c_void_p, C.c_int, _dp, C.c_int, C.POINTER(BoltHier), C.c_double, C.c_double,
                                     _dp, _i32p]),
    "bolt_source_grid": (C.c_int, [C.c_void_p, C.c_int, _dp, C.c_int, C.POINTER(BoltHier), C.c_double,
                                   C.c_double, _dp, _dp, _i32p]),
    "bolt_cl": (C.c_int, [C.c_void_p, C.c_int, _dp, _dp, _dp, C.c_int, _ip, C.c_int, _dp, _dp, _dp]),
    "bolt_cl_pipeline": (C.c_int, [C.c_void_p, C.c_int, _dp, C.c_int, C.POINTER(BoltHier), C.c_double,
                                   C.c_double, _ip, C.c_int, _dp, _dp, _dp, _i32p]),
    "bolt_plin": (C.c_int, [C.c_void_p, C.c_int, _dp, C.c_int, C.POINTER(BoltHier), C.c_double, C.c_double,
                            C.c_double, _dp, _i32p]),
    "bolt_last_stats": (C.c_int, [C.c_void_p, _i64p]),
    "bolt_adjoint_check": (C.c_int, [C.c_void_p, C.c_int, C.c_double, C.POINTER(BoltHier), C.c_double, C.c_double,
                                     _dp]),
    "bolt_fp64_peak": (C.c_int, [C.c_int, _dp]),
    "bolt_set_dense_x": (C.c_int, [C.c_void_p, C.c_double]),
    "bolt_set_land_stride": (C.c_int, [C.c_void_p, C.c_int]),
    "bolt_sph_j_moment": (C.c_int, [C.c_void_p, C.c_int, C.c_double, _dp, C.c_int, _dp]),
    "bolt_moment_table_build": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, _ip]),
    "bolt_moment_table_eval": (C.c_int, [C.c_void_p, C.c_int, _dp, C.c_int, _dp]),
    "bolt_moment_table_free": (C.c_int, [C.c_void_p, C.c_int]),
    "bolt_filon": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, _dp]),
    "bolt_filon_piecewise": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _dp, _dp, _dp, _dp, C.c_int, _dp, _dp]),
    "bolt_filon_batched": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _dp, _dp, _dp, _dp, C.c_int, _dp, _dp]),
    "bolt_source_grid_static": (C.c_int, [C.POINTER(BoltParams), C.POINTER(BoltGrid), C.c_int, _dp, _dp, _dp,
                                          C.c_int, C.POINTER(BoltHier), C.c_double, C.c_double, C.c_void_p,
                                          C.c_void_p, C.c_void_p, C.c_void_p, C.c_char_p, C.c_int]),
    "bolt_engine_create": (C.c_int, [C.POINTER(BoltEngineCfg), C.POINTER(C.c_void_p)]),
    "bolt_engine_destroy": (None, [C.c_void_p]),
    "bolt_engine_last_error": (C.c_char_p, [C.c_void_p]),
    "bolt_engine_submit": (C.c_int, [C.c_void_p, C.POINTER(BoltRequest), _i64p]),
    "bolt_engine_wait": (C.c_int, [C.c_void_p, C.c_int64, C.c_double, _ip, _dp, C.c_char_p, C.c_int]),
    "bolt_request_run": (C.c_int, [C.c_void_p, C.POINTER(BoltRequest), C.c_char_p, C.c_int]),
    "bolt_cl_vjp": (C.c_int, [C.c_void_p, C.POINTER(BoltRequest), _dp, _dp, _dp, _dp, C.c_char_p, C.c_int]),
    "bolt_plin_vjp": (C.c_int, [C.c_void_p, C.POINTER(BoltRequest), _dp, _dp, C.c_char_p, C.c_int]),
    "bolt_engine_stats": (C.c_int, [C.c_void_p, _i64p]),
}

_lib = None


def load(build_if_missing: bool = True):
    """Loads (and if needed builds) the in-tree library."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path) or not _build.up_to_date():
        if not build_if_missing:
            raise ImportError(f"libbolt_gb300.so is missing at {path}; run the build first")
        _build.build()
    L = C.CDLL(path)
    for name, (res, args) in EXPORTS.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def dptr(a):
    return a.ctypes.data_as(_dp) if a is not None else None


def iptr(a):
    return a.ctypes.data_as(_ip) if a is not None else None


def i32ptr(a):
    return a.ctypes.data_as(_i32p) if a is not None else None
