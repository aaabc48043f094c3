"""ctypes front end of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline / reference arm, never by the product package.  It supplies the results the GPU path is compared with; it
is not the thing measured or shipped.

Every function takes flat numpy storage buffers plus (M, N, K, ld*) in the reference's layout
(versions.hpp:43-45):
    TSMTTSM  C[n*ldc+m] = alpha * sum_k A[k*lda+m] * B[k*ldb+n] + beta * C[n*ldc+m]
    TSMM     C[r*ldc+n] = alpha * sum_m A[r*lda+m] * B[n*ldb+m] + beta * C[r*ldc+n]
Complex buffers are numpy complex64/complex128 (interleaved re, im).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

_SUFFIX = {np.dtype(np.float32): "s", np.dtype(np.float64): "d",
           np.dtype(np.complex64): "c", np.dtype(np.complex128): "z"}


# Where the reference tree is mounted when the reference's own kernels are compiled (the cubins
# in oracle/_ref are built only where it exists and are used as prebuilt files elsewhere).
REFERENCE_TREE = os.environ.get("SKINNY_REFERENCE_TREE", "/root/reference")


def build() -> str:
    """Compile the oracle with its Makefile (gcc + OpenMP) and the runner of the reference's
    kernels; where the reference tree exists, also the reference's kernels (oracle/_ref).
    Returns the oracle library's path."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    if os.path.isdir(os.path.join(REFERENCE_TREE, "tsmttsm")):
        subprocess.run(["make", "-s", "-j5", "-C", _HERE, "ref", f"REF={REFERENCE_TREE}"], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        _lib = ctypes.CDLL(_LIB_PATH)
        i64, vp, ci = ctypes.c_int64, ctypes.c_void_p, ctypes.c_int
        for op in ("tsmttsm", "tsmm"):
            for s in "sdcz":
                f = getattr(_lib, f"orc_{op}_{s}")
                f.argtypes = [i64, i64, i64, vp, i64, vp, vp, i64, vp, vp, i64, ci]
                f.restype = None
        _lib.orc_tsmttsm_pq.argtypes = [i64, i64, i64, vp, i64, vp, vp, i64, vp, vp, i64, ci]
        for nm in ("orc_tsmttsm_exact_d", "orc_tsmttsm_exact_z", "orc_tsmm_exact_d", "orc_tsmm_exact_z"):
            getattr(_lib, nm).argtypes = [i64, i64, i64, vp, i64, vp, i64, vp, vp, i64, ci]
        _lib.orc_dot_exact.argtypes = [i64, vp, i64, vp, i64, vp, vp]
        dp = ctypes.POINTER(ctypes.c_double)
        for nm in ("orc_pq_fast2sum", "orc_pq_gen2sum", "orc_pq_fma2mult"):
            getattr(_lib, nm).argtypes = [ctypes.c_double, ctypes.c_double, dp, dp]
        _lib.orc_pq_accu.argtypes = [ctypes.c_double] * 4 + [dp, dp]
        _lib.orc_pq_axpy2.argtypes = [ctypes.c_double] * 4 + [dp, dp]
        _lib.orc_pq_scale2.argtypes = [ctypes.c_double] * 3 + [dp, dp]
        _lib.orc_max_threads.restype = ctypes.c_int
    return _lib


def _ptr(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.c_void_p)


def _scalar(v, dt):
    return np.array([v], dtype=dt)


def max_threads() -> int:
    return lib().orc_max_threads()


def tsmttsm(M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, nthreads=0, acc="native"):
    """C (in/out) <- alpha * A^T B + beta * C.  acc='pq' selects double-double accumulation."""
    dt = A.dtype
    al, be = _scalar(alpha, dt), _scalar(beta, dt)
    if acc == "pq":
        assert dt == np.float64
        fn = lib().orc_tsmttsm_pq
    else:
        fn = getattr(lib(), "orc_tsmttsm_" + _SUFFIX[dt])
    fn(M, N, K, _ptr(A), lda, _ptr(al), _ptr(B), ldb, _ptr(be), _ptr(C), ldc, nthreads)
    return C


def tsmm(M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, nthreads=0):
    """C (in/out) <- alpha * A B + beta * C; A is C allowed (in place, lda == ldc)."""
    dt = A.dtype
    al, be = _scalar(alpha, dt), _scalar(beta, dt)
    fn = getattr(lib(), "orc_tsmm_" + _SUFFIX[dt])
    fn(M, N, K, _ptr(A), lda, _ptr(al), _ptr(B), ldb, _ptr(be), _ptr(C), ldc, nthreads)
    return C


def _exact(kind, M, N, K, A, lda, B, ldb, lds, nrows, nthreads):
    cplx = np.iscomplexobj(A)
    A64 = A.astype(np.complex128 if cplx else np.float64)
    B64 = B.astype(np.complex128 if cplx else np.float64)
    hi = np.zeros(nrows * lds, dtype=A64.dtype)
    lo = np.zeros_like(hi)
    fn = getattr(lib(), f"orc_{kind}_exact_{'z' if cplx else 'd'}")
    fn(M, N, K, _ptr(A64), lda, _ptr(B64), ldb, _ptr(hi), _ptr(lo), lds, nthreads)
    return hi, lo


def tsmttsm_exact(M, N, K, A, lda, B, ldb, lds=None, nthreads=0):
    """Exact S = A^T B rounded to double-double; returns (hi, lo) with S[n*lds+m]."""
    lds = M if lds is None else lds
    return _exact("tsmttsm", M, N, K, A, lda, B, ldb, lds, N, nthreads)


def tsmm_exact(M, N, K, A, lda, B, ldb, lds=None, nthreads=0):
    """Exact S = A B rounded to double-double; returns (hi, lo) with S[r*lds+n]."""
    lds = N if lds is None else lds
    return _exact("tsmm", M, N, K, A, lda, B, ldb, lds, K, nthreads)


def dot_exact(a: np.ndarray, b: np.ndarray):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    hi, lo = ctypes.c_double(), ctypes.c_double()
    lib().orc_dot_exact(len(a), _ptr(a), 1, _ptr(b), 1, ctypes.byref(hi), ctypes.byref(lo))
    return hi.value, lo.value


def pq(name, *args):
    """Call one PseudoQuad primitive (fast2sum, gen2sum, fma2mult, accu, axpy2, scale2)."""
    s, t = ctypes.c_double(), ctypes.c_double()
    getattr(lib(), "orc_pq_" + name)(*[float(a) for a in args], ctypes.byref(s), ctypes.byref(t))
    return s.value, t.value


def normwise_error(C_hat, S_hi, S_lo, absprod):
    """||C_hat - S||_F / ||absprod||_F with S = S_hi + S_lo (differences taken in double-double
    order: (C_hat - S_hi) - S_lo, exact when C_hat is close to S_hi)."""
    d = (C_hat.astype(S_hi.dtype) - S_hi) - S_lo
    den = np.linalg.norm(absprod.ravel())
    num = np.linalg.norm(d.ravel())
    return float(num / den) if den > 0 else float(num)
