"""ctypes binding of libskewgpu.so (the C ABI in include/skewgpu.h).

The shared library is the product; this module only declares its signatures.
There is no fallback: if the library cannot be loaded, importing skewgpu fails.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libskewgpu.so")

SKEW_OK = 0
SKEW_NOT_SKEW = 1
SKEW_NO_CONVERGENCE = 2
SKEW_BAD_ARG = 3
SKEW_CUDA_ERROR = 4
SKEW_SINGULAR = 5
SKEW_UNSUPPORTED = 6
SKEW_NO_MEMORY = 7
SKEW_FALLBACK_USED = 8
SKEW_TIMEOUT = 9

_vp = ctypes.c_void_p
_i64 = ctypes.c_int64
_int = ctypes.c_int

# name -> (restype, argtypes); the authoritative list of exported entry points
SIGNATURES = {
    "skew_create": (_int, [ctypes.POINTER(_vp)]),
    "skew_destroy": (_int, [_vp]),
    "skew_set_stream": (_int, [_vp, _vp]),
    "skew_status_string": (ctypes.c_char_p, [_int]),
    "skew_version": (_int, []),
    "skew_hessenberg_d": (_int, [_vp, _vp, _i64, _i64, _vp, _vp, _vp]),
    "skew_logabspf_d": (_int, [_vp, _vp, _i64, _i64, _vp, _vp, _int, _vp]),
    "skew_logabspf_grad_d": (_int, [_vp, _vp, _i64, _i64, _vp, _vp, _vp, _i64, _vp]),
    "skew_eigvals_d": (_int, [_vp, _vp, _i64, _i64, _vp, _vp]),
    "skew_eigvals_noalloc_d": (_int, [_vp, _i64, _i64, _vp, _vp, _vp]),
    "skew_eigen_d": (_int, [_vp, _vp, _i64, _i64, _vp, _vp, _vp, _i64, _vp]),
    "skew_exp_d": (_int, [_vp, _vp, _i64, _i64, _vp, _i64, _vp]),
    "skew_cis_d": (_int, [_vp, _vp, _i64, _i64, _vp, _i64, _vp]),
    "skew_batch_plan_create": (_int, [_vp, ctypes.POINTER(_i64), _i64, ctypes.POINTER(_vp)]),
    "skew_batch_plan_destroy": (_int, [_vp]),
    "skew_batch_logabspf_d": (_int, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "skew_batch_logabspf_host_d": (_int, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "skew_batch_eigvals_d": (_int, [_vp, _vp, _vp, _vp]),
    "skew_batch_eigen_d": (_int, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "skew_batch_exp_d": (_int, [_vp, _vp, _vp, _vp]),
    "skew_batch_cis_d": (_int, [_vp, _vp, _vp, _vp]),
    "skew_batch_exp_vjp_d": (_int, [_vp, _vp, _vp, _vp, _vp]),
    "skew_exp_vjp_d": (_int, [_vp, _vp, _i64, _i64, _vp, _vp, _i64, _vp]),
    "skew_hessenberg_z": (_int, [_vp, _vp, _i64, _i64, _vp, _vp, _vp, _vp]),
    "skew_eigvals_z": (_int, [_vp, _vp, _i64, _i64, _vp, _vp]),
    "skew_eigen_z": (_int, [_vp, _vp, _i64, _i64, _vp, _vp, _i64, _vp]),
    "skew_exp_z": (_int, [_vp, _vp, _i64, _i64, _vp, _i64, _vp]),
    "skew_exp_vjp_z": (_int, [_vp, _vp, _i64, _i64, _vp, _vp, _i64, _vp]),
    "skew_batch_eigen_z": (_int, [_vp, _vp, _i64, _i64, _vp, _vp, _vp]),
    "skew_batch_exp_z": (_int, [_vp, _vp, _i64, _i64, _vp, _vp]),
    "skew_batch_exp_vjp_z": (_int, [_vp, _vp, _i64, _i64, _vp, _vp, _vp]),
    "skew_func_d": (_int, [_vp, _vp, _i64, _i64, _int, _vp, _i64, _vp]),
    "skew_tridiag_eigvals_d": (_int, [_vp, _vp, _i64, _vp, _vp]),
    "skew_tridiag_eigen_d": (_int, [_vp, _vp, _i64, _vp, _vp, _vp, _i64, _vp]),
    "skew_tridiag_func_d": (_int, [_vp, _vp, _i64, _int, _vp, _i64, _vp]),
    "skew_tridiag_eigvals_z": (_int, [_vp, _vp, _vp, _i64, _vp, _vp]),
    "skew_tridiag_eigen_z": (_int, [_vp, _vp, _vp, _i64, _vp, _vp, _i64, _vp]),
    "skew_eigvals_irange_d": (_int, [_vp, _vp, _i64, _i64, _i64, _i64, _vp, _vp]),
    "skew_eigvals_interval_d": (_int, [_vp, _vp, _i64, _i64, ctypes.c_double, ctypes.c_double, _vp, _vp, _vp]),
    "skew_eigvals_interval_z": (_int, [_vp, _vp, _i64, _i64, ctypes.c_double, ctypes.c_double, _vp, _vp, _vp]),
    "skew_batch_func_d": (_int, [_vp, _vp, _int, _vp, _vp]),
    "skew_func_z": (_int, [_vp, _vp, _i64, _i64, _int, _vp, _i64, _vp]),
    "skew_batch_func_z": (_int, [_vp, _vp, _i64, _i64, _int, _vp, _vp]),
    "skew_svdvals_d": (_int, [_vp, _vp, _i64, _i64, _vp, _vp]),
    "skew_svd_d": (_int, [_vp, _vp, _i64, _i64, _vp, _vp, _vp, _vp, _vp, _i64, _vp]),
    "skew_svdvals_z": (_int, [_vp, _vp, _i64, _i64, _vp, _vp]),
    "skew_svd_z": (_int, [_vp, _vp, _i64, _i64, _vp, _vp, _vp, _i64, _vp]),
    "skew_tridiag_svdvals_d": (_int, [_vp, _vp, _i64, _vp, _vp]),
    "skew_tridiag_svd_d": (_int, [_vp, _vp, _i64, _vp, _vp, _vp, _vp, _vp, _i64, _vp]),
    "skew_tridiag_svdvals_z": (_int, [_vp, _vp, _vp, _i64, _vp, _vp]),
    "skew_tridiag_svd_z": (_int, [_vp, _vp, _vp, _i64, _vp, _vp, _vp, _i64, _vp]),
    "skew_logabspf_z": (_int, [_vp, _vp, _i64, _i64, _vp, _vp, _int, _vp]),
    "skew_pfaffian_z": (_int, [_vp, _vp, _i64, _i64, _vp, _int, _vp]),
    "skew_batch_logabspf_z": (_int, [_vp, _vp, _i64, _i64, _vp, _vp, _vp, _int, _vp]),
    "skew_batch_logabspf_host_z": (_int, [_vp, _vp, _i64, _i64, _vp, _vp, _vp, _int, _vp]),
    "skew_measure_fp64_peak": (_int, [_vp, ctypes.POINTER(ctypes.c_double)]),
    "skew_measure_fp64_pipes": (_int, [_vp, ctypes.POINTER(ctypes.c_double)]),
    "skew_tuning_set": (_int, [_vp, ctypes.c_char_p, ctypes.c_int64]),
    "skew_tuning_set_list": (_int, [_vp, ctypes.c_char_p, ctypes.POINTER(ctypes.c_int64), _int]),
    "skew_tuning_get": (_int, [_vp, ctypes.c_char_p, ctypes.POINTER(ctypes.c_int64), _int, ctypes.POINTER(_int)]),
    "skew_tuning_reset": (_int, [_vp]),
    "skew_tuning_load": (_int, [_vp, ctypes.c_char_p]),
    "skew_tuning_source": (ctypes.c_char_p, [_vp]),
    "skew_tuning_key": (ctypes.c_char_p, [_int]),
    "skew_tuning_file_get": (_int, [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p,
                                    ctypes.POINTER(ctypes.c_int64), _int, ctypes.POINTER(_int)]),
}

_lib = None


class SkewError(RuntimeError):
    def __init__(self, status: int, where: str = ""):
        self.status = status
        msg = status_string(status) if _lib is not None else str(status)
        super().__init__(f"{where}: {msg} (status {status})" if where else f"{msg} (status {status})")


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"libskewgpu.so is not built ({LIB_PATH}); run __graft_entry__.build()")
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def status_string(status: int) -> str:
    return load().skew_status_string(int(status)).decode()


def check(status: int, where: str = "") -> None:
    if status != SKEW_OK:
        raise SkewError(status, where)
