"""CPU tests that pin the oracle before anything is checked against it.

* every golden integer case (test.cu fixture design) is reproduced bit-exactly by the plain-loop
  restatement, for TSMTTSM / TSMM, real / complex, Gram and in-place modes;
* the exact super-accumulator matches fractions.Fraction on wide-range data and on the
  numeric_tests.cu cancellation KAT;
* the double-double restatement's primitives satisfy their error-free-transformation identities
  (PseudoQuad.cuh:10-31,66-75,96-108) and its TSMTTSM recovers the KAT where plain FP64 fails.
"""
from fractions import Fraction

import numpy as np
import pytest

import common
from oracle import oracle as O


@pytest.mark.parametrize("case", list(common.int_cases()), ids=lambda c: c["id"])
def test_golden_integer_cases(case):
    c = case
    A, B, C = c["A"].copy(), c["B"].copy(), c["C"].copy()
    if c["self"] and c["op"] == "tsmttsm":
        B = A
    if c["self"] and c["op"] == "tsmm":
        A = C
    fn = O.tsmttsm if c["op"] == "tsmttsm" else O.tsmm
    fn(c["M"], c["N"], c["K"], A, c["lda"], 1.0, B, c["ldb"], float(c["beta"]), C, c["ldc"])
    assert np.array_equal(C, c["exp"])


@pytest.mark.parametrize("case", [c for c in common.int_cases() if not c["cplx"] and c["op"] == "tsmttsm"][:12],
                         ids=lambda c: c["id"])
def test_golden_integer_cases_float32_and_dd(case):
    c = case
    A32, B32, C32 = (x.astype(np.float32) for x in (c["A"], c["B"], c["C"]))
    if c["self"]:
        B32 = A32
    O.tsmttsm(c["M"], c["N"], c["K"], A32, c["lda"], 1.0, B32, c["ldb"], float(c["beta"]), C32, c["ldc"])
    assert np.array_equal(C32.astype(np.float64), c["exp"])
    Cd = c["C"].copy()
    O.tsmttsm(c["M"], c["N"], c["K"], c["A"], c["lda"], 1.0, c["A"] if c["self"] else c["B"], c["ldb"],
              float(c["beta"]), Cd, c["ldc"], acc="pq")
    assert np.array_equal(Cd, c["exp"])


def test_exact_accumulator_matches_fraction():
    rng = np.random.default_rng(7)
    n = 3000
    a = rng.uniform(-1, 1, n) * np.ldexp(1.0, rng.integers(-300, 300, n))
    b = rng.uniform(-1, 1, n) * np.ldexp(1.0, rng.integers(-300, 300, n))
    hi, lo = O.dot_exact(a, b)
    ex = sum(Fraction(float(x)) * Fraction(float(y)) for x, y in zip(a, b))
    assert hi == float(ex)
    assert lo == float(ex - Fraction(hi))


def test_exact_accumulator_is_thread_count_independent():
    rng = np.random.default_rng(3)
    M, N, K = 5, 3, 4000
    A = common.spread(rng, K * M)
    B = common.spread(rng, K * N)
    h1, l1 = O.tsmttsm_exact(M, N, K, A, M, B, N, nthreads=1)
    h8, l8 = O.tsmttsm_exact(M, N, K, A, M, B, N, nthreads=8)
    assert np.array_equal(h1, h8) and np.array_equal(l1, l8)
    for j in (0, 7, 14):
        m, n = j % M, j // M
        ex = sum(Fraction(float(A[k * M + m])) * Fraction(float(B[k * N + n])) for k in range(K))
        assert h1[n * M + m] == float(ex)


def test_kat_exact_value():
    a, b, d = common.kat()
    hi, lo = O.dot_exact(a, b)
    assert hi == d["exact_hi"] and lo == d["exact_lo"]
    ex = Fraction(int(d["exact_numerator"]), int(d["exact_denominator"]))
    assert ex == (len(a) - 4) * Fraction(0.1) ** 2  # all four big products cancel


@pytest.mark.parametrize("nthreads", [1, 8, 64])
def test_kat_double_double_beats_fp64(nthreads):
    """numeric_tests.cu:58-61 runs the KAT through SPECSMALL<double,double> and
    SPECSMALL<double,PseudoQuad>.  The two +-2^124 products keep the running sum near 2^124 while
    the 0.01 terms arrive, so no order of double-double accumulation is exact (106 bits cannot
    span 2^124 .. 2^-7); double-double still keeps most of the small terms, plain FP64 none, and
    both stay inside the normwise bound 8 sqrt(K) u relative to sum |a_i b_i|."""
    a, b, d = common.kat()
    N = len(a)
    ex = d["exact_hi"]
    out_pq, out_d = np.zeros(1), np.zeros(1)
    O.tsmttsm(1, 1, N, a, 1, 1.0, b, 1, 0.0, out_pq, 1, acc="pq", nthreads=nthreads)
    O.tsmttsm(1, 1, N, a, 1, 1.0, b, 1, 0.0, out_d, 1, nthreads=nthreads)
    err_pq, err_d = abs(out_pq[0] - ex), abs(out_d[0] - ex)
    assert err_d > 0.9 * abs(ex)        # plain FP64 loses (nearly) everything
    assert err_pq < 0.5 * err_d          # double-double keeps most of it
    absdot = float(np.abs(a) @ np.abs(b))
    assert err_pq / absdot <= common.tol(np.float64, N)


def test_kat_without_outer_pair_is_recovered_by_double_double():
    """The same vector with only the +-2^62 * 0.1 cancellation: now 106 bits span the range and
    double-double accumulation must return the exact value to within a few ulps."""
    a, b, d = common.kat()
    N = len(a)
    a[0] = a[N - 1] = b[0] = b[N - 1] = 0.1
    hi, lo = O.dot_exact(a, b)
    out = np.zeros(1)
    O.tsmttsm(1, 1, N, a, 1, 1.0, b, 1, 0.0, out, 1, acc="pq")
    assert abs(out[0] - hi) <= 2 * np.spacing(hi)


def test_pq_primitives_error_free():
    rng = np.random.default_rng(11)
    for _ in range(2000):
        x, y = rng.normal() * 2.0 ** rng.integers(-40, 40), rng.normal() * 2.0 ** rng.integers(-40, 40)
        s, t = O.pq("gen2sum", x, y)
        assert Fraction(s) + Fraction(t) == Fraction(x) + Fraction(y)
        if abs(x) >= abs(y):
            s, t = O.pq("fast2sum", x, y)
            assert Fraction(s) + Fraction(t) == Fraction(x) + Fraction(y)
        s, t = O.pq("fma2mult", x, y)
        assert Fraction(s) + Fraction(t) == Fraction(x) * Fraction(y)


def test_pq_axpy2_and_accu_are_compensated():
    """axpy2 (PseudoQuad.cuh:96-108) is a compensated multiply-add: over a random chain its error
    relative to sum |a b| is far below plain FP64 accumulation's, though not at the 2^-104 level
    (a cancelling step can lose about u * |a b| because a*b is not a double)."""
    rng = np.random.default_rng(0)
    a, b = rng.uniform(-1, 1, 2000), rng.uniform(-1, 1, 2000)
    cs, ct, p = 0.0, 0.0, 0.0
    for x, y in zip(a, b):
        cs, ct = O.pq("axpy2", cs, ct, x, y)
        p += x * y
    ex = sum(Fraction(float(x)) * Fraction(float(y)) for x, y in zip(a, b))
    sab = float(sum(abs(Fraction(float(x)) * Fraction(float(y))) for x, y in zip(a, b)))
    err_pq = float(abs(Fraction(cs) + Fraction(ct) - ex)) / sab
    err_d = float(abs(Fraction(p) - ex)) / sab
    assert err_pq < 2.0 ** -58 and err_pq < err_d / 20
    s, t = O.pq("accu", 1.0, 1e-20, 3.0, -2e-20)
    assert Fraction(s) + Fraction(t) == Fraction(4.0) + Fraction(1e-20) - Fraction(2e-20) or \
        abs(float(Fraction(s) + Fraction(t) - (Fraction(4.0) + Fraction(1e-20) - Fraction(2e-20)))) < 1e-35


@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.complex64, np.complex128])
def test_plain_oracle_within_bound_of_exact(dtype):
    rng = np.random.default_rng(1)
    M, N, K = 4, 6, 20000
    A = common.uniform(rng, K * M, dtype)
    B = common.uniform(rng, K * N, dtype)
    C0 = common.uniform(rng, N * M, dtype)
    C = C0.copy()
    O.tsmttsm(M, N, K, A, M, 1.0, B, N, 0.5, C, M)
    exp, den = common.tsmttsm_expected(M, N, K, A, M, B, N, C0, M, 1.0, 0.5)
    assert common.normwise(C, exp, den) <= common.tol(dtype, K)
    Ct = common.uniform(rng, 300 * N, dtype)
    Ct0 = Ct.copy()
    At = common.uniform(rng, 300 * M, dtype)
    Bt = common.uniform(rng, M * N, dtype)
    O.tsmm(M, N, 300, At, M, 1.0, Bt, M, 0.5, Ct, N)
    exp, den = common.tsmm_expected(M, N, 300, At, M, Bt, M, Ct0, N, 1.0, 0.5)
    assert common.normwise(Ct, exp, den) <= common.tol(dtype, M)
