"""Shared helpers for the tests: golden fixtures, seeded inputs and error metrics."""
from __future__ import annotations

import json
import math
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

UNIT_ROUNDOFF = {np.dtype(np.float32): 2.0 ** -24, np.dtype(np.float64): 2.0 ** -53,
                 np.dtype(np.complex64): 2.0 ** -24, np.dtype(np.complex128): 2.0 ** -53}


def int_cases():
    """Yields dicts for every golden integer case (tests/golden/make_golden.py)."""
    z = np.load(os.path.join(GOLDEN, "int_cases.npz"))
    keys = sorted({k.split("_")[0] for k in z.files})
    for k in keys:
        op, M, N, K, lda, ldb, ldc, beta, self_mode, cplx = (int(v) for v in z[k + "_meta"])
        def arr(name):
            a = z[k + "_" + name]
            if cplx:
                a = a.astype(np.float64)
                return (a[0::2] + 1j * a[1::2]).astype(np.complex128)
            return a.astype(np.float64)
        yield dict(id=k, op="tsmttsm" if op == 0 else "tsmm", M=M, N=N, K=K, lda=lda, ldb=ldb, ldc=ldc,
                   beta=beta, self=self_mode, cplx=cplx, A=arr("A"), B=arr("B"), C=arr("C"), exp=arr("exp"))


def kat():
    with open(os.path.join(GOLDEN, "kat_cancellation.json")) as f:
        d = json.load(f)
    N = d["N"]
    a = np.full(N, 0.1)
    b = np.full(N, 0.1)
    big = float(2 ** 62)
    for i in d["big_index_a"]:
        a[i] = big
    a[41234] = -big
    b[0] = big
    b[N - 1] = -big
    return a, b, d


def uniform(rng, n, dtype):
    dt = np.dtype(dtype)
    if dt.kind == "c":
        real = np.float32 if dt == np.complex64 else np.float64
        return (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(dt)
    return rng.uniform(-1, 1, n).astype(dt)


def spread(rng, n):
    """s * 2^e, s in U[1,2), random sign, e uniform in [-20, 20] (the precision workload)."""
    s = rng.uniform(1, 2, n)
    e = rng.integers(-20, 21, n)
    sg = np.where(rng.integers(0, 2, n) == 0, -1.0, 1.0)
    return sg * np.ldexp(s, e)


def tol(dtype, K):
    """Normwise bound 8 * sqrt(K) * u of the working precision."""
    return 8.0 * math.sqrt(max(K, 1)) * UNIT_ROUNDOFF[np.dtype(dtype)]


def _fill(rows, width, ld, S, ahi, C0, alpha, beta):
    exp = C0.astype(S.dtype).copy()
    den = np.zeros(len(exp))
    e2, d2 = exp.reshape(rows, ld), den.reshape(rows, ld)
    s2, a2, c2 = S.reshape(rows, ld), ahi.reshape(rows, ld), C0.reshape(rows, ld)
    e2[:, :width] = alpha * s2[:, :width] + (beta * c2[:, :width] if beta != 0 else 0)
    d2[:, :width] = abs(alpha) * a2[:, :width] + (abs(beta) * np.abs(c2[:, :width]) if beta != 0 else 0)
    return exp, den


def tsmttsm_expected(M, N, K, A, lda, B, ldb, C0, ldc, alpha, beta):
    """(expected C, normwise denominator array) from the exact oracle, in float64/complex128."""
    from oracle import oracle as O
    hi, lo = O.tsmttsm_exact(M, N, K, A, lda, B, ldb, lds=ldc)
    ahi, _ = O.tsmttsm_exact(M, N, K, np.abs(A).astype(np.float64), lda, np.abs(B).astype(np.float64), ldb, lds=ldc)
    return _fill(N, M, ldc, hi + lo, ahi, C0, alpha, beta)


def tsmm_expected(M, N, K, A, lda, B, ldb, C0, ldc, alpha, beta):
    from oracle import oracle as O
    hi, lo = O.tsmm_exact(M, N, K, A, lda, B, ldb, lds=ldc)
    ahi, _ = O.tsmm_exact(M, N, K, np.abs(A).astype(np.float64), lda, np.abs(B).astype(np.float64), ldb, lds=ldc)
    return _fill(K, N, ldc, hi + lo, ahi, C0, alpha, beta)


def normwise(got, exp, den, mask=None):
    d = (got.astype(exp.dtype) - exp)
    if mask is not None:
        d = d[mask]
        den = den[mask]
    nd = np.linalg.norm(den)
    return float(np.linalg.norm(d) / nd) if nd > 0 else float(np.linalg.norm(d))


def c_mask_tsmttsm(M, N, ldc):
    m = np.zeros(N * ldc, dtype=bool)
    for n in range(N):
        m[n * ldc: n * ldc + M] = True
    return m


def c_mask_tsmm(N, K, ldc):
    m = np.zeros(K * ldc, dtype=bool)
    for r in range(K):
        m[r * ldc: r * ldc + N] = True
    return m
