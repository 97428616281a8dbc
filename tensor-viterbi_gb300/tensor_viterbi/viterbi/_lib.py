"""ctypes binding of libtv_gb300.so (the C ABI declared in include/tv_gb300.h).

The library is the only implementation: if it is missing or fails to load,
every call raises.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import pathlib
import threading

import numpy as np

LIB_PATH = pathlib.Path(__file__).resolve().parents[2] / "libtv_gb300.so"

TV_OK = 0
TV_EINVAL = -1
TV_ESHORT = -2
TV_ERANGE = -3
TV_ENONFINITE = -4
TV_ETOOBIG = -5
TV_ENOMEM = -6
TV_ECUDA = -7
TV_EINTERNAL = -8
TV_ENODEV = -9
TV_ETIMEOUT = -10
TV_ENONPOS = -11

# Argument errors surface as ValueError (the caller passed something the
# decoder cannot accept); runtime failures as RuntimeError.
_VALUE_ERRORS = {TV_EINVAL, TV_ESHORT, TV_ERANGE, TV_ENONFINITE, TV_ETOOBIG}

_lock = threading.Lock()
_lib = None

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_lp = C.POINTER(C.c_int64)

EXPORTS = {
    "tv_last_error": (C.c_char_p, []),
    "tv_decode_tensor_viterbi_cuda": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int64, _dp, _dp, _dp, _dp, _dp, _ip, _ip, _dp]),
    "tv_model_create": (C.c_int, [C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp, C.POINTER(C.c_void_p)]),
    "tv_model_destroy": (C.c_int, [C.c_void_p]),
    "tv_decode": (C.c_int, [C.c_void_p, _ip, C.c_int64, _ip, _dp]),
    "tv_decode_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]),
    "tv_decode_batch": (C.c_int, [C.c_void_p, C.c_int, _lp, _ip, _ip, _dp]),
    "tv_decode_batch_device": (C.c_int, [C.c_void_p, C.c_int, _lp, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "tv_model_last_launches": (C.c_int64, [C.c_void_p]),
    "tv_model_set_path": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "tv_model_last_path": (C.c_int, [C.c_void_p]),
    "tv_model_batch_threads": (C.c_int, [C.c_void_p]),
    "tv_model_batch_grid": (C.c_int, [C.c_void_p]),
    "tv_model_drop_partial": (C.c_int, [C.c_void_p, C.c_int64, C.c_int]),
    "tv_grid_plan_info": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p]),
    "tv_model_set_timing": (C.c_int, [C.c_void_p, C.c_int]),
    "tv_model_kernel_ms": (C.c_double, [C.c_void_p]),
    "tv_step_floor": (C.c_int, [C.c_int, C.c_int, C.c_int64, _dp]),
    "tv_fp64_peak": (C.c_int, [_dp]),
    "tv_fb_last_kernel_ms": (C.c_double, []),
    "tv_fb": (C.c_int, [C.c_int, C.c_int64, C.c_int, C.c_int] + [_dp] * 11),
    "tv_decode_device_static": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.c_void_p]),
    "tv_gaussian_loglik": (C.c_int, [C.c_void_p, C.c_int64, C.c_int, _dp, _dp, C.c_void_p, C.c_void_p]),
    "tv_model_create_gaussian": (C.c_int, [C.c_int, C.c_int, C.c_int64, _dp, _dp, _dp, _dp, _dp, _dp, _dp,
                                           C.POINTER(C.c_void_p)]),
    "tv_server_create": (C.c_void_p, [C.c_int64, C.c_int]),
    "tv_server_destroy": (C.c_int, [C.c_void_p]),
    "tv_server_submit": (C.c_int64, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int64, _dp, _dp, _dp, _dp, _dp, _ip]),
    "tv_server_submit_gaussian": (C.c_int64, [C.c_void_p, C.c_int, C.c_int, C.c_int64, _dp, _dp, _dp, _dp, _dp, _dp,
                                              _dp]),
    "tv_server_poll": (C.c_int, [C.c_void_p, C.c_int64, _ip, _dp, _dp]),
    "tv_server_wait": (C.c_int, [C.c_void_p, C.c_int64, _ip, _dp, _dp]),
    "tv_server_stats": (C.c_int, [C.c_void_p, _lp]),
}

# Size of the fixed device scratch behind tv_decode_device_static.
TV_STATIC_SCRATCH_BYTES = 32 << 20

TV_PATH_AUTO = 0
TV_PATH_CTA = 1
TV_PATH_GRID = 2
TV_PATH_GRID_L2 = 3


def lib():
    """Load libtv_gb300.so once; raise if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise RuntimeError(
                    f"[native] GB300 decoder library not built: {LIB_PATH} is missing. "
                    "Run `python tensor-viterbi_gb300/build.py` (or __graft_entry__.build())."
                )
            h = C.CDLL(str(LIB_PATH))
            for name, (res, args) in EXPORTS.items():
                fn = getattr(h, name)
                fn.restype = res
                fn.argtypes = args
            _lib = h
    return _lib


def check(rc: int) -> None:
    if rc == TV_OK:
        return
    msg = lib().tv_last_error().decode(errors="replace")
    if rc in _VALUE_ERRORS:
        raise ValueError(f"[native] {msg} (status {rc})")
    raise RuntimeError(f"[native] {msg} (status {rc})")


def dptr(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def iptr(a: np.ndarray):
    return a.ctypes.data_as(_ip)


def lptr(a: np.ndarray):
    return a.ctypes.data_as(_lp)
