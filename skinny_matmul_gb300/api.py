"""Host-side mirror of the reference's launcher interface, over the C ABI.

The reference exposes one launcher per kernel variant with the shape (versions.hpp:43-45)
    bool f(blockCount, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc)
and its harness keeps them in a list of (function, name) pairs (versions.hpp:48-177,
test.cu:251-301).  `launchers(op, dtype)` returns the same kind of list for this library, and
`tsmttsm` / `tsmm` / `svqb` are the stream-aware calls of include/skinny.h.  Device buffers are
torch CUDA tensors (flat storage in the reference layout) or raw device addresses (int).
"""
from __future__ import annotations

import ctypes
from typing import Callable, List, Tuple

from . import lib as L

_ACC = {"native": L.ACC_NATIVE, "dd": L.ACC_DD, "split": L.ACC_SPLIT, "auto": L.ACC_AUTO}


def _dtype_code(t) -> int:
    import torch
    m = {torch.float32: L.R32, torch.float64: L.R64, torch.complex64: L.C32, torch.complex128: L.C64}
    if t.dtype not in m:
        raise TypeError(f"unsupported dtype {t.dtype}")
    return m[t.dtype]


def _scalar(v, code):
    if code == L.R32:
        return ctypes.c_float(float(v))
    if code == L.R64:
        return ctypes.c_double(float(v))
    v = complex(v)
    return (L.c32 if code == L.C32 else L.c64)(v.real, v.imag)


def _ptr(x):
    if x is None:
        return None
    if isinstance(x, int):
        return x
    return x.data_ptr()


def _stream(stream):
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


class Handle:
    """Owns a skinny_handle (device, per-stream workspaces, autotune table)."""

    def __init__(self, device: int = 0):
        self.lib = L.load()
        h = ctypes.c_void_p()
        L.check(self.lib.skinny_create(ctypes.byref(h), device))
        self.h = h
        self.device = device

    def close(self):
        if self.h:
            self.lib.skinny_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check_device(self):
        return L.check(self.lib.skinny_check_device(self.h))

    def set_wait_limit(self, polls: int):
        """Poll limit of the bounded device-side waits (include/skinny.h skinny_set_wait_limit)."""
        return L.check(self.lib.skinny_set_wait_limit(self.h, polls))

    def _product(self, fn, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, acc, stream, dtype):
        code = dtype if dtype is not None else _dtype_code(A if not isinstance(A, int) else C)
        al, be = _scalar(alpha, code), _scalar(beta, code)
        st = fn(self.h, code, _ACC[acc], M, N, K, _ptr(A), lda, ctypes.byref(al), _ptr(B), ldb,
                ctypes.byref(be), _ptr(C), ldc, _stream(stream))
        return L.check(st)

    def tsmttsm(self, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, acc="native", stream=None, dtype=None,
                conj=False):
        """C[n*ldc+m] = alpha * sum_k A[k*lda+m] B[k*ldb+n] + beta * C[n*ldc+m]; conj=True takes the
        conjugate of A (C = alpha A^H B + beta C)."""
        fn = self.lib.skinny_tsmttsm_conj if conj else self.lib.skinny_tsmttsm
        return self._product(fn, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, acc, stream, dtype)

    def tsmm(self, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, acc="native", stream=None, dtype=None):
        """C[r*ldc+n] = alpha * sum_m A[r*lda+m] B[n*ldb+m] + beta * C[r*ldc+n]  (A may be C)."""
        return self._product(self.lib.skinny_tsmm, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc,
                             acc, stream, dtype)

    def autotune(self, op, dtype, M, N, K, acc="auto", stream=None):
        """Measure launch shapes (and, for FP64 'auto', split vs CUDA-core) for (op, dtype, acc,
        M, N) on scratch operands of K rows; the handle then uses the fastest for that key.
        op: 'tsmttsm' | 'tsmm'; dtype: 'float32' | 'float64' | 'complex64' | 'complex128'."""
        code = {"float32": L.R32, "float64": L.R64, "complex64": L.C32, "complex128": L.C64}[dtype]
        return L.check(self.lib.skinny_autotune(self.h, 0 if op == "tsmttsm" else 1, code, _ACC[acc],
                                                M, N, K, _stream(stream)))

    def tune_export(self) -> str:
        n = ctypes.c_size_t()
        L.check(self.lib.skinny_tune_export(self.h, None, 0, ctypes.byref(n)))
        buf = ctypes.create_string_buffer(n.value)
        L.check(self.lib.skinny_tune_export(self.h, buf, n.value, ctypes.byref(n)))
        return buf.value.decode()

    def tune_import(self, text: str):
        return L.check(self.lib.skinny_tune_import(self.h, text.encode()))

    def cholqr(self, K, M, X, ldx, passes=2, gram_acc="auto", orth_err=True, stream=None):
        """In-place CholQR (passes=1) / CholQR2 (passes=2) of X (K x M, FP64); returns
        ||Q^T Q - I||_F when orth_err."""
        err = ctypes.c_double(-1.0)
        L.check(self.lib.skinny_cholqr(self.h, _ACC[gram_acc], K, M, _ptr(X), ldx, passes,
                                       ctypes.byref(err) if orth_err else None, _stream(stream)))
        return err.value if orth_err else None

    def group(self, items, dtype=None, stream=None):
        """One grouped launch (skinny_group) of small products of one dtype.  `items` are dicts
        with op ('tsmttsm' | 'tsmm'), M, N, K, A, lda, B, ldb, C, ldc and optional alpha (1),
        beta (0); A, B, C device tensors or addresses.  dtype: 'float32' | 'float64' |
        'complex64' | 'complex128' (default: from the first item's A)."""
        if not items:
            return L.OK
        code = _DT[dtype] if dtype is not None else _dtype_code(items[0]["A"])
        arr = (L.GroupItem * len(items))()
        for g, it in zip(arr, items):
            g.op = _OPS[it["op"]]
            g.M, g.N, g.K = it["M"], it["N"], it["K"]
            g.A, g.lda = _ptr(it["A"]), it["lda"]
            g.B, g.ldb = _ptr(it["B"]), it["ldb"]
            g.C, g.ldc = _ptr(it["C"]), it["ldc"]
            a, b = complex(it.get("alpha", 1.0)), complex(it.get("beta", 0.0))
            g.alpha[0], g.alpha[1], g.beta[0], g.beta[1] = a.real, a.imag, b.real, b.imag
        return L.check(self.lib.skinny_group(self.h, code, arr, len(items), _stream(stream)))

    def svqb(self, K, M, X, ldx, gram_acc="split", orth_err=True, stream=None):
        """In-place SVQB of X (K x M, FP64, or complex FP64 with the Hermitian Gram); returns
        ||Q^H Q - I||_F when orth_err."""
        err = ctypes.c_double(-1.0)
        fn = self.lib.skinny_svqb_z if _dtype_code(X) == L.C64 else self.lib.skinny_svqb
        L.check(fn(self.h, _ACC[gram_acc], K, M, _ptr(X), ldx, ctypes.byref(err) if orth_err else None,
                   _stream(stream)))
        return err.value if orth_err else None


_default: dict = {}


def default_handle(device: int | None = None) -> Handle:
    if device is None:
        import torch
        device = torch.cuda.current_device()
    if device not in _default:
        _default[device] = Handle(device)
    return _default[device]


def tsmttsm(M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, acc="native", stream=None, handle=None):
    return (handle or default_handle()).tsmttsm(M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, acc, stream)


def tsmm(M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, acc="native", stream=None, handle=None):
    return (handle or default_handle()).tsmm(M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, acc, stream)


def svqb(K, M, X, ldx, gram_acc="split", orth_err=True, stream=None, handle=None):
    return (handle or default_handle()).svqb(K, M, X, ldx, gram_acc, orth_err, stream)


def svqb_host_dd(X, K, M, threads=0, orth_err=True):
    """Double-double SVQB on the host (skinny_svqb_host_dd): X a host float64 array of K x M
    (row-major); returns (Q, ||Q^T Q - I||_F or None).  Needs no GPU."""
    import numpy as np
    Xc = np.ascontiguousarray(X, dtype=np.float64).reshape(-1)
    if Xc.size < K * M:
        raise ValueError("X holds fewer than K * M values")
    Q = np.empty(K * M, dtype=np.float64)
    err = ctypes.c_double(-1.0)
    L.check(L.load().skinny_svqb_host_dd(Xc.ctypes.data, Q.ctypes.data, K, M, threads,
                                         ctypes.byref(err) if orth_err else None))
    return Q, (err.value if orth_err else None)


_REF_SUFFIX = {"float32": "s", "float64": "d", "complex64": "c", "complex128": "z", "dd": "dd"}


def launchers(op: str, dtype: str) -> List[Tuple[Callable, str]]:
    """Reference-shaped launchers for `op` ("tsmttsm" | "tsmm") and `dtype`, as (fn, name) pairs
    like getEnabledTSMTTSMVersions / getEnabledTSMMVersions (versions.hpp:48-177).
    fn(blockCount, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc) -> bool, on the legacy default
    stream.  A, B, C are device addresses (int) or tensors."""
    lib = L.load()
    sfx = _REF_SUFFIX[dtype]
    raw = getattr(lib, f"skinny_{op}_{sfx}")
    cplx = sfx in ("c", "z")
    ct = {"s": ctypes.c_float, "d": ctypes.c_double, "dd": ctypes.c_double, "c": L.c32, "z": L.c64}[sfx]

    def fn(blockCount, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc):
        conv = (lambda v: ct(complex(v).real, complex(v).imag)) if cplx else (lambda v: ct(v))
        P = ctypes.POINTER(ct)
        return bool(raw(blockCount, M, N, K, ctypes.cast(_ptr(A), P), lda, conv(alpha),
                        ctypes.cast(_ptr(B), P), ldb, conv(beta), ctypes.cast(_ptr(C), P), ldc))

    return [(fn, f"GB300_{op.upper()}_{sfx.upper()}")]


_OPS = {"tsmttsm": L.OP_TSMTTSM, "tsmm": L.OP_TSMM, "svqb": L.OP_SVQB}
_DT = {"float32": L.R32, "float64": L.R64, "complex64": L.C32, "complex128": L.C64}


class Server:
    """Request loop with continuous batching (skinny_server_* in include/skinny.h).

    Requests carry HOST numpy buffers (keep them alive until the ticket completes; pinned memory
    overlaps transfers) or, with device=True, device tensors resident in HBM.  handle=None runs
    the scheduler in dry mode (no device work)."""

    def __init__(self, handle: Handle | None, mem_budget_bytes: int, num_streams: int = 4,
                 max_inflight: int = 16, group_bytes: int | None = None, group_max: int = 512):
        self.lib = L.load()
        s = ctypes.c_void_p()
        L.check(self.lib.skinny_server_create(ctypes.byref(s), handle.h if handle else None,
                                              int(mem_budget_bytes), num_streams, max_inflight))
        self.s = s
        self._keep = {}
        if group_bytes is not None:
            self.set_grouping(group_bytes, group_max)

    def set_grouping(self, max_request_bytes: int, max_group: int = 512):
        """Requests up to max_request_bytes (TSMTTSM / TSMM, native or auto, M, N <= 64) run in
        grouped launches of up to max_group; 0 turns grouping off."""
        return L.check(self.lib.skinny_server_set_grouping(self.s, int(max_request_bytes), int(max_group)))

    def submit(self, op, dtype, M, N, K, A, lda, B=None, ldb=0, C=None, ldc=0, alpha=1.0, beta=0.0,
               acc="native", device=False):
        """Queue a request; returns its ticket.  A, B, C are host arrays (numpy) or addresses; with
        device=True they are device tensors (or device addresses) resident in HBM, used in place."""
        def addr(x):
            if x is None:
                return None
            if isinstance(x, int):
                return x
            if hasattr(x, "data_ptr"):
                return x.data_ptr()
            return x.ctypes.data
        r = L.Request()
        r.op, r.dtype, r.acc = _OPS[op], _DT[dtype], _ACC[acc]
        r.M, r.N, r.K = M, N, K
        r.A, r.lda, r.B, r.ldb, r.C, r.ldc = addr(A), lda, addr(B), ldb, addr(C), ldc
        a, b = complex(alpha), complex(beta)
        r.alpha[0], r.alpha[1], r.beta[0], r.beta[1] = a.real, a.imag, b.real, b.imag
        r.device = 1 if device else 0
        t = ctypes.c_uint64()
        st = self.lib.skinny_server_submit(self.s, ctypes.byref(r), ctypes.byref(t))
        if st == L.OK:
            self._keep[t.value] = (A, B, C)
        return st, t.value

    def poll(self, ticket):
        res = ctypes.c_int(-1)
        st = self.lib.skinny_server_poll(self.s, ticket, ctypes.byref(res))
        return st, res.value

    def wait(self, ticket, timeout_s=60.0):
        res = ctypes.c_int(-1)
        st = self.lib.skinny_server_wait(self.s, ticket, ctypes.byref(res), timeout_s)
        if st == L.OK:
            self._keep.pop(ticket, None)
        return st, res.value

    def drain(self, timeout_s=600.0):
        return L.check(self.lib.skinny_server_drain(self.s, timeout_s))

    def stats(self) -> dict:
        s = L.ServerStats()
        L.check(self.lib.skinny_server_stats_get(self.s, ctypes.byref(s)))
        return {f: getattr(s, f) for f, _ in L.ServerStats._fields_}

    def close(self):
        if self.s:
            self.lib.skinny_server_destroy(self.s)
            self.s = None
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
