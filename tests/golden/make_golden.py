"""Generates the committed golden fixtures under tests/golden/ (run once; outputs are committed).

1. int_cases.npz -- the reference harness's fixture design (test.cu:65-103, 247-276): entries are
   small integers drawn from {-2..2}, leading dimensions padded by 0..4, K random, beta in {0, 1},
   both aliasing modes (TSMTTSM A == B Gram; TSMM C == A in place).  Every partial sum is then an
   exactly representable integer, so every correct implementation is bit-exact regardless of its
   summation order (test.cu:172-174 compares with !=).  Expected outputs are computed here with
   Python integers, independently of the oracle and of the library.
2. kat_cancellation.json -- the precision known-answer test of numeric_tests.cu:22-73: N = 111113,
   a_i = b_i = fl(0.1) except a[0] = a[1234] = a[N-1] = 2^62, a[41234] = -2^62, b[0] = 2^62,
   b[N-1] = -2^62.  The exact dot product is computed here with fractions.Fraction (the
   reference's printed "should be" value at numeric_tests.cu:71 is approximate and not used).

Usage:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
from fractions import Fraction

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SEED = 20241203


def _tsmttsm_int(M, N, K, A, lda, B, ldb, C0, ldc, beta):
    """Exact integer C[n*ldc+m] = sum_k A[k*lda+m] B[k*ldb+n] + beta*C0 (alpha = 1)."""
    Ai = A.astype(object)
    Bi = B.astype(object)
    out = C0.astype(object).copy()
    for n in range(N):
        for m in range(M):
            s = 0
            for k in range(K):
                s += Ai[k * lda + m] * Bi[k * ldb + n]
            out[n * ldc + m] = s + (beta * C0[n * ldc + m] if beta != 0 else 0)
    return out


def _tsmm_int(M, N, K, A, lda, B, ldb, C0, ldc, beta):
    """Exact integer C[r*ldc+n] = sum_m A[r*lda+m] B[n*ldb+m] + beta*C0 (alpha = 1)."""
    out = C0.astype(object).copy()
    for r in range(K):
        row = [int(A[r * lda + m]) for m in range(M)]
        for n in range(N):
            s = sum(row[m] * int(B[n * ldb + m]) for m in range(M))
            out[r * ldc + n] = s + (beta * int(C0[r * ldc + n]) if beta != 0 else 0)
    return out


def _cplx_split(z):
    return np.stack([z.real, z.imag], -1).ravel()


def make_int_cases():
    rng = np.random.default_rng(SEED)
    cases = {}
    shapes = [(1, 1), (2, 2), (3, 3), (4, 4), (8, 8), (5, 7), (4, 16), (16, 4), (8, 32), (16, 16),
              (32, 32), (1, 8), (13, 3)]
    idx = 0
    for op in ("tsmttsm", "tsmm"):
        for (M, N) in shapes:
            for self_mode in (0, 1):
                if op == "tsmttsm" and self_mode and M != N:
                    continue
                for beta in (0, 1):
                    for cplx in (0, 1):
                        if cplx and (M * N > 256):
                            continue
                        lda = M + int(rng.integers(0, 5))
                        if op == "tsmttsm":
                            ldb = N + int(rng.integers(0, 5))
                            ldc = M + int(rng.integers(0, 5))
                            K = int(rng.integers(1, 600 if M * N <= 64 else 160))
                            if self_mode:
                                ldb = lda
                            nA, nB, nC = K * lda, K * ldb, N * ldc
                        else:
                            ldb = M + int(rng.integers(0, 5))
                            ldc = (max(N + int(rng.integers(0, 5)), M) if self_mode else N + int(rng.integers(0, 5)))
                            K = int(rng.integers(1, 200))
                            if self_mode:
                                lda = ldc  # in place: A is C (test.cu:131)
                            nA, nB, nC = K * lda, ldb * N, K * ldc
                        def draw(n):
                            if cplx:
                                return rng.integers(-2, 3, n) + 1j * rng.integers(-2, 3, n)
                            return rng.integers(-2, 3, n).astype(np.int64)
                        A = draw(nA)
                        B = draw(nB)
                        C0 = draw(nC)
                        if op == "tsmttsm" and self_mode:
                            B = A
                        if op == "tsmm" and self_mode:
                            A = C0
                        if cplx:
                            # exact complex integer arithmetic through Python ints
                            if op == "tsmttsm":
                                exp = np.zeros(nC, dtype=complex)
                                for n in range(N):
                                    for m in range(M):
                                        s = 0
                                        for k in range(K):
                                            s += complex(A[k * lda + m]) * complex(B[k * ldb + n])
                                        exp[n * ldc + m] = s + (beta * C0[n * ldc + m] if beta else 0)
                                for i in range(nC):
                                    if (i % ldc) >= M:
                                        exp[i] = C0[i]
                            else:
                                exp = C0.copy()
                                for r in range(K):
                                    for n in range(N):
                                        s = 0
                                        for m in range(M):
                                            s += complex(A[r * lda + m]) * complex(B[n * ldb + m])
                                        exp[r * ldc + n] = s + (beta * C0[r * ldc + n] if beta else 0)
                            # all values are integers well below 2^53: complex128 holds them exactly
                            exp_arr = _cplx_split(exp).astype(np.int64)
                            A_arr, B_arr, C_arr = (_cplx_split(x).astype(np.int8) for x in (A, B, C0))
                        else:
                            f = _tsmttsm_int if op == "tsmttsm" else _tsmm_int
                            exp = f(M, N, K, A, lda, B, ldb, C0, ldc, beta)
                            exp_arr = np.array(exp, dtype=np.int64)
                            A_arr, B_arr, C_arr = (x.astype(np.int8) for x in (A, B, C0))
                        key = f"c{idx:03d}"
                        idx += 1
                        cases[key + "_meta"] = np.array(
                            [0 if op == "tsmttsm" else 1, M, N, K, lda, ldb, ldc, beta, self_mode, cplx],
                            dtype=np.int64)
                        cases[key + "_A"] = A_arr
                        cases[key + "_B"] = B_arr
                        cases[key + "_C"] = C_arr
                        cases[key + "_exp"] = exp_arr
    np.savez_compressed(os.path.join(HERE, "int_cases.npz"), **cases)
    return idx


def kat_vectors():
    """The cancellation vectors of numeric_tests.cu:23-53."""
    N = 111113
    a = np.full(N, 0.1)
    b = np.full(N, 0.1)
    big = float(2 ** 62)
    a[0] = big
    a[1234] = big
    a[41234] = -big
    a[N - 1] = big
    b[0] = big
    b[N - 1] = -big
    return a, b


def make_kat():
    a, b = kat_vectors()
    exact = sum(Fraction(float(x)) * Fraction(float(y)) for x, y in zip(a, b))
    hi = float(exact)
    lo = float(exact - Fraction(hi))
    out = {"N": len(a), "big_index_a": [0, 1234, 41234, len(a) - 1], "big_index_b": [0, len(a) - 1],
           "exact_numerator": str(exact.numerator), "exact_denominator": str(exact.denominator),
           "exact_hi": hi, "exact_lo": lo}
    with open(os.path.join(HERE, "kat_cancellation.json"), "w") as f:
        json.dump(out, f, indent=1)
    return out


if __name__ == "__main__":
    n = make_int_cases()
    k = make_kat()
    print(f"{n} integer cases; KAT exact = {k['exact_hi']!r} + {k['exact_lo']!r}")
