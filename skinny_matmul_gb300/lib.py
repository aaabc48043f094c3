"""ctypes binding of the C ABI in include/skinny.h (libskinny.so).

This is the binding a Python caller of the reference's launchers would add: every symbol of the
header, with its exact argument types.  There is no fallback: if the shared library is missing
or fails to load, importing the product raises.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

LIB_PATH = _build.LIB

R32, R64, C32, C64 = 0, 1, 2, 3
ACC_NATIVE, ACC_DD, ACC_SPLIT, ACC_AUTO = 0, 1, 2, 3
OK, UNSUPPORTED, BAD_ARG, NO_MEM, TIMEOUT, DEVICE_ERROR, NOT_READY = range(7)
STATUS_NAMES = ["SKINNY_OK", "SKINNY_UNSUPPORTED", "SKINNY_BAD_ARG", "SKINNY_NO_MEM",
                "SKINNY_TIMEOUT", "SKINNY_DEVICE_ERROR", "SKINNY_NOT_READY"]


class c32(ctypes.Structure):
    _fields_ = [("x", ctypes.c_float), ("y", ctypes.c_float)]


class c64(ctypes.Structure):
    _fields_ = [("x", ctypes.c_double), ("y", ctypes.c_double)]


class Request(ctypes.Structure):
    """skinny_request (include/skinny.h)."""
    _fields_ = [("op", ctypes.c_int), ("dtype", ctypes.c_int), ("acc", ctypes.c_int),
                ("M", ctypes.c_int64), ("N", ctypes.c_int64), ("K", ctypes.c_int64),
                ("A", ctypes.c_void_p), ("lda", ctypes.c_int64), ("B", ctypes.c_void_p), ("ldb", ctypes.c_int64),
                ("C", ctypes.c_void_p), ("ldc", ctypes.c_int64),
                ("alpha", ctypes.c_double * 2), ("beta", ctypes.c_double * 2), ("device", ctypes.c_int32)]


class ServerStats(ctypes.Structure):
    """skinny_server_stats (include/skinny.h)."""
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64), ("failed", ctypes.c_uint64),
                ("rejected", ctypes.c_uint64), ("p50_latency_us", ctypes.c_double),
                ("p99_latency_us", ctypes.c_double), ("mean_latency_us", ctypes.c_double),
                ("bytes", ctypes.c_double), ("busy_seconds", ctypes.c_double),
                ("peak_bytes_in_use", ctypes.c_uint64), ("max_inflight_seen", ctypes.c_uint64),
                ("grouped", ctypes.c_uint64), ("group_launches", ctypes.c_uint64)]


class GroupItem(ctypes.Structure):
    """skinny_group_item (include/skinny.h)."""
    _fields_ = [("op", ctypes.c_int), ("M", ctypes.c_int64), ("N", ctypes.c_int64), ("K", ctypes.c_int64),
                ("A", ctypes.c_void_p), ("lda", ctypes.c_int64), ("B", ctypes.c_void_p), ("ldb", ctypes.c_int64),
                ("C", ctypes.c_void_p), ("ldc", ctypes.c_int64),
                ("alpha", ctypes.c_double * 2), ("beta", ctypes.c_double * 2)]


OP_TSMTTSM, OP_TSMM, OP_SVQB = 0, 1, 2


class SkinnyError(RuntimeError):
    def __init__(self, status: int, detail: str = ""):
        self.status = status
        name = STATUS_NAMES[status] if 0 <= status < len(STATUS_NAMES) else str(status)
        super().__init__(f"{name}: {detail}" if detail else name)


_lib = None

# (name, restype, argtypes) for every entry point declared in include/skinny.h
_i64, _vp, _i, _sz = ctypes.c_int64, ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t
_PROD = [_vp, _i, _i, _i64, _i64, _i64, _vp, _i64, _vp, _vp, _i64, _vp, _vp, _i64, _vp]


def _ref_sig(T, HT):
    return [_sz, _i, _i, _i, ctypes.POINTER(T), _i, HT, ctypes.POINTER(T), _i, HT, ctypes.POINTER(T), _i]


SIGNATURES = {
    "skinny_create": (_i, [ctypes.POINTER(_vp), _i]),
    "skinny_destroy": (_i, [_vp]),
    "skinny_status_string": (ctypes.c_char_p, [_i]),
    "skinny_last_error": (ctypes.c_char_p, []),
    "skinny_check_device": (_i, [_vp]),
    "skinny_set_wait_limit": (_i, [_vp, ctypes.c_uint32]),
    "skinny_kernel_launches": (ctypes.c_uint64, []),
    "skinny_tsmttsm": (_i, _PROD),
    "skinny_tsmttsm_conj": (_i, _PROD),
    "skinny_tsmm": (_i, _PROD),
    "skinny_svqb": (_i, [_vp, _i, _i64, _i64, _vp, _i64, _vp, _vp]),
    "skinny_cholqr": (_i, [_vp, _i, _i64, _i64, _vp, _i64, _i, _vp, _vp]),
    "skinny_svqb_z": (_i, [_vp, _i, _i64, _i64, _vp, _i64, _vp, _vp]),
    "skinny_svqb_host_dd": (_i, [_vp, _vp, _i64, _i, _i, _vp]),
    "skinny_autotune": (_i, [_vp, _i, _i, _i, _i64, _i64, _i64, _vp]),
    "skinny_tune_export": (_i, [_vp, ctypes.c_char_p, _sz, ctypes.POINTER(_sz)]),
    "skinny_tune_import": (_i, [_vp, ctypes.c_char_p]),
    "skinny_server_create": (_i, [ctypes.POINTER(_vp), _vp, ctypes.c_uint64, _i, _i]),
    "skinny_server_submit": (_i, [_vp, ctypes.POINTER(Request), ctypes.POINTER(ctypes.c_uint64)]),
    "skinny_server_poll": (_i, [_vp, ctypes.c_uint64, ctypes.POINTER(_i)]),
    "skinny_server_wait": (_i, [_vp, ctypes.c_uint64, ctypes.POINTER(_i), ctypes.c_double]),
    "skinny_server_drain": (_i, [_vp, ctypes.c_double]),
    "skinny_server_stats_get": (_i, [_vp, ctypes.POINTER(ServerStats)]),
    "skinny_server_destroy": (_i, [_vp]),
    "skinny_server_set_grouping": (_i, [_vp, ctypes.c_uint64, ctypes.c_int32]),
    "skinny_group": (_i, [_vp, _i, ctypes.POINTER(GroupItem), ctypes.c_int32, _vp]),
    "skinny_tsmttsm_d_static": (_i, [_i64, _i64, _i64, _vp, _i64, ctypes.c_double, _vp, _i64,
                                     ctypes.c_double, _vp, _i64, _vp]),
    "skinny_tsmttsm_d_static_check": (_i, [_vp]),
    "skinny_tsmttsm_s": (_i, _ref_sig(ctypes.c_float, ctypes.c_float)),
    "skinny_tsmttsm_d": (_i, _ref_sig(ctypes.c_double, ctypes.c_double)),
    "skinny_tsmttsm_c": (_i, _ref_sig(c32, c32)),
    "skinny_tsmttsm_z": (_i, _ref_sig(c64, c64)),
    "skinny_tsmttsm_dd": (_i, _ref_sig(ctypes.c_double, ctypes.c_double)),
    "skinny_tsmm_s": (_i, _ref_sig(ctypes.c_float, ctypes.c_float)),
    "skinny_tsmm_d": (_i, _ref_sig(ctypes.c_double, ctypes.c_double)),
    "skinny_tsmm_c": (_i, _ref_sig(c32, c32)),
    "skinny_tsmm_z": (_i, _ref_sig(c64, c64)),
    "skinny_tsmm_dd": (_i, _ref_sig(ctypes.c_double, ctypes.c_double)),
}


def load(path: str | None = None):
    """Load libskinny.so (built by build.build()) and bind every entry point."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"libskinny.so not found at {p}: run skinny_matmul_gb300.build.build() first")
    lib = ctypes.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def last_error() -> str:
    return load().skinny_last_error().decode()


def check(status: int):
    if status != OK:
        raise SkinnyError(status, last_error())
    return status
