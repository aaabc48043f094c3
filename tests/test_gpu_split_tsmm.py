"""GPU parity tests of the FP64 / complex FP64 split-precision TSMM (tcgen05) against the oracle.

Bars: golden integer cases bit-exact; random data within 8 sqrt(M) u normwise (u = 2^-53) of the
exact oracle and, as the split products are formed exactly and rounded a few times, within 8e-16."""
import numpy as np
import pytest

import common

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


CASES = [c for c in common.int_cases() if c["op"] == "tsmm" and
         ((not c["cplx"] and c["M"] <= 64 and c["N"] <= 64) or (c["cplx"] and c["M"] <= 32 and c["N"] <= 32))]


@pytest.mark.parametrize("case", CASES, ids=lambda c: c["id"])
@pytest.mark.parametrize("single", [False, True], ids=["fp64", "fp32"])
def test_split_tsmm_golden_bit_exact(handle, case, single):
    """The integer fixtures, in FP64 / complex FP64 and in FP32 / complex FP32 storage (their
    values and results are exact in both)."""
    c = case
    dt = (np.complex64 if c["cplx"] else np.float32) if single else (np.complex128 if c["cplx"] else np.float64)
    A, B, C = dev(c["A"].astype(dt)), dev(c["B"].astype(dt)), dev(c["C"].astype(dt))
    if c["self"]:
        A = C
    handle.tsmm(c["M"], c["N"], c["K"], A, c["lda"], 1.0, B, c["ldb"], float(c["beta"]), C, c["ldc"], acc="split")
    got = host(C).astype(np.complex128 if c["cplx"] else np.float64)
    assert np.array_equal(got, c["exp"])


SHAPES = [(1, 1), (2, 2), (4, 4), (8, 8), (16, 16), (32, 32), (4, 16), (16, 4), (8, 32), (3, 5), (17, 9), (32, 1),
          (64, 64), (64, 8), (8, 64), (33, 47)]


@pytest.mark.parametrize("M,N", SHAPES)
@pytest.mark.parametrize("inplace", [False, True])
def test_split_tsmm_uniform(handle, M, N, inplace):
    if inplace and M != N:
        pytest.skip("in place needs M == N here")
    rng = np.random.default_rng(M * 100 + N)
    K = 20011
    lda, ldb, ldc = M, M + 1, N
    if inplace:
        lda = ldc = M
    A = rng.uniform(-1, 1, K * lda)
    B = rng.uniform(-1, 1, N * ldb)
    C0 = A.copy() if inplace else rng.uniform(-1, 1, K * ldc)
    Cd = dev(C0)
    Ad = Cd if inplace else dev(A)
    handle.tsmm(M, N, K, Ad, lda, 1.5, dev(B), ldb, -0.5, Cd, ldc, acc="split")
    got = host(Cd)
    exp, den = common.tsmm_expected(M, N, K, C0 if inplace else A, lda, B, ldb, C0, ldc, 1.5, -0.5)
    err = common.normwise(got, exp, den, common.c_mask_tsmm(N, K, ldc))
    assert err <= min(common.tol(np.float64, M), 8e-16), err


@pytest.mark.parametrize("M,N", [(1, 1), (2, 2), (4, 4), (8, 8), (16, 16), (4, 16), (16, 4), (3, 7), (32, 32),
                                 (8, 32)])
@pytest.mark.parametrize("inplace", [False, True])
def test_split_tsmm_complex(handle, M, N, inplace):
    if inplace and M != N:
        pytest.skip("in place needs M == N here")
    rng = np.random.default_rng(7 + M * 13 + N)
    K = 10007
    lda, ldb, ldc = M, M, N
    A = common.uniform(rng, K * lda, np.complex128)
    B = common.uniform(rng, N * ldb, np.complex128)
    C0 = A.copy() if inplace else common.uniform(rng, K * ldc, np.complex128)
    alpha, beta = 1.0 + 0.5j, 0.5 - 0.25j
    Cd = dev(C0)
    Ad = Cd if inplace else dev(A)
    handle.tsmm(M, N, K, Ad, lda, alpha, dev(B), ldb, beta, Cd, ldc, acc="split")
    got = host(Cd)
    exp, den = common.tsmm_expected(M, N, K, C0 if inplace else A, lda, B, ldb, C0, ldc, alpha, beta)
    err = common.normwise(got, exp, den, common.c_mask_tsmm(N, K, ldc))
    assert err <= min(common.tol(np.complex128, M), 8e-16), err


@pytest.mark.parametrize("dt", [np.float32, np.complex64])
@pytest.mark.parametrize("M,N", [(1, 1), (4, 4), (8, 8), (16, 16), (4, 16), (8, 32), (3, 7), (32, 32), (64, 64),
                                 (17, 9), (40, 8)])
@pytest.mark.parametrize("inplace", [False, True])
def test_split_tsmm_fp32(handle, dt, M, N, inplace):
    """FP32 and complex FP32 storage on the split kernel: exact products, FP64-accurate sums, one
    rounding to FP32 at the end -- within 2^-23 normwise of the exact result (the native FP32
    kernels are held to 8 sqrt(M) 2^-24); odd leading dimensions take the unvectorised paths."""
    if inplace and M != N:
        pytest.skip("in place needs M == N here")
    cplx = dt == np.complex64
    if cplx and max(M, N) > 32:
        M, N = min(M, 32), min(N, 32)
    rng = np.random.default_rng(11 + M * 7 + N)
    K = 9001
    lda, ldb, ldc = (M, M + 1, N) if not inplace else (M, M, M)
    if M == 3:
        lda, ldc = M + 2, N + 1  # 4-byte rows that are not 16-byte multiples
    A = common.uniform(rng, K * lda, dt)
    B = common.uniform(rng, N * ldb, dt)
    C0 = A.copy() if inplace else common.uniform(rng, K * ldc, dt)
    alpha, beta = (1.0 + 0.5j, 0.5 - 0.25j) if cplx else (1.5, -0.5)
    Cd = dev(C0)
    Ad = Cd if inplace else dev(A)
    handle.tsmm(M, N, K, Ad, lda, alpha, dev(B), ldb, beta, Cd, ldc, acc="split")
    got = host(Cd)
    exp, den = common.tsmm_expected(M, N, K, C0 if inplace else A, lda, B, ldb, C0, ldc, alpha, beta)
    err = common.normwise(got, exp, den, common.c_mask_tsmm(N, K, ldc))
    assert err <= 2.0 ** -23, err


def test_split_tsmm_wide_exponents_and_zero_rows(handle):
    rng = np.random.default_rng(3)
    M = N = 16
    K = 30000
    A = common.spread(rng, K * M)
    A[: 5 * M] = 0.0  # all-zero rows
    B = common.spread(rng, M * N)
    C0 = common.spread(rng, K * N)
    Cd = dev(C0)
    handle.tsmm(M, N, K, dev(A), M, 1.0, dev(B), M, 0.25, Cd, N, acc="split")
    got = host(Cd)
    exp, den = common.tsmm_expected(M, N, K, A, M, B, M, C0, N, 1.0, 0.25)
    assert common.normwise(got, exp, den) <= 8e-16


def test_split_tsmm_unaligned_and_padded(handle):
    rng = np.random.default_rng(4)
    M, N, K = 8, 8, 5003
    for lda, off in ((M + 3, 0), (M, 1), (3 * M + 20, 1)):
        A = rng.uniform(-1, 1, K * lda + 1)
        B = rng.uniform(-1, 1, M * N)
        C0 = rng.uniform(-1, 1, K * N)
        Cd = dev(C0)
        Ad = dev(A)
        handle.tsmm(M, N, K, Ad[off:], lda, 1.0, dev(B), M, 1.0, Cd, N, acc="split")
        exp, den = common.tsmm_expected(M, N, K, A[off:].copy(), lda, B, M, C0, N, 1.0, 1.0)
        assert common.normwise(host(Cd), exp, den) <= 8e-16, (lda, off)


def test_split_tsmm_small_k(handle):
    rng = np.random.default_rng(5)
    for K in (1, 127, 128, 129, 255):
        M, N = 8, 4
        A = rng.uniform(-1, 1, K * M)
        B = rng.uniform(-1, 1, M * N)
        Cd = dev(np.zeros(K * N))
        handle.tsmm(M, N, K, dev(A), M, 1.0, dev(B), M, 0.0, Cd, N, acc="split")
        exp, den = common.tsmm_expected(M, N, K, A, M, B, M, np.zeros(K * N), N, 1.0, 0.0)
        assert common.normwise(host(Cd), exp, den) <= 8e-16, K


@pytest.mark.parametrize("cplx,M,N", [(True, 64, 64), (True, 32, 64), (True, 64, 16), (True, 40, 33),
                                      (False, 128, 128), (False, 96, 64), (False, 70, 20), (False, 16, 100)])
def test_split_tsmm_wide_in_passes(handle, cplx, M, N):
    """Real widths above 64 run as passes (output-column chunks; contraction chunks accumulate
    through beta)."""
    rng = np.random.default_rng(M * 7 + N + cplx)
    K = 6007
    dt = np.complex128 if cplx else np.float64
    lda, ldb, ldc = M + 1, M, N + 2
    A = common.uniform(rng, K * lda, dt)
    B = common.uniform(rng, N * ldb, dt)
    C0 = common.uniform(rng, K * ldc, dt)
    alpha, beta = (0.5 + 0.25j, -0.75 + 0.5j) if cplx else (1.25, -0.5)
    Cd = dev(C0)
    handle.tsmm(M, N, K, dev(A), lda, alpha, dev(B), ldb, beta, Cd, ldc, acc="split")
    got = host(Cd)
    exp, den = common.tsmm_expected(M, N, K, A, lda, B, ldb, C0, ldc, alpha, beta)
    err = common.normwise(got, exp, den, common.c_mask_tsmm(N, K, ldc))
    assert err <= min(common.tol(dt, M), 8e-16), err


def test_split_tsmm_wide_in_place_unsupported(handle):
    from skinny_matmul_gb300 import lib as L
    M = 40
    K = 1000
    X = dev(np.zeros(K * M, np.complex128))
    B = dev(np.zeros(M * M, np.complex128))
    with pytest.raises(L.SkinnyError):
        handle.tsmm(M, M, K, X, M, 1.0, B, M, 0.0, X, M, acc="split")


def test_split_tsmm_epilogue_window_no_overflow(handle):
    """A row and column whose level-2..5 sum H lies just below 2^35 in magnitude while the
    lower levels add in the same direction: shifting H up to bit 62 and adding the low part
    overflowed int64 once (the SVQB transform of a Gaussian block hit it).  Exact value from the
    oracle."""
    a = np.array([-0.0902333034774286, 0.9953960347960409, -2.0001290059485535, 1.1617594199348404,
                  0.028492030066136674, 0.09951610977610051, -0.5629304941495062, -0.5286079153781488,
                  -0.06524758134155434, 2.6990741536801366, -1.2709225246596088, 0.7713573735580164,
                  -0.6003361654324079, 1.3004598145928816, -1.444973049978174, -0.6231094244429115])
    b = np.array([-0.00011886051243768427, 3.243606984224829e-05, -0.00021251367167326099,
                  -0.0003335254616945151, -0.000156368179871508, 4.834772800842875e-06,
                  -0.0004869401572375484, 0.00041763952392900086, 7.545508081615978e-05,
                  -0.0001768818370975454, 0.00024901494173812844, -0.00036403177288671997,
                  -0.00016018322106158998, -2.026052523593613e-05, -5.568237286745128e-05,
                  0.00028435164789257793])
    M, N = 16, 16
    K = 300
    rng = np.random.default_rng(0)
    A = rng.standard_normal((K, M))
    A[137] = a
    B = rng.standard_normal((N, M)) * 1e-4
    B[13] = b
    Cd = dev(np.zeros(K * N))
    handle.tsmm(M, N, K, dev(A.ravel()), M, 1.0, dev(B.ravel()), M, 0.0, Cd, N, acc="split")
    got = host(Cd)
    exp, den = common.tsmm_expected(M, N, K, A.ravel(), M, B.ravel(), M, np.zeros(K * N), N, 1.0, 0.0)
    assert common.normwise(got, exp, den) <= 8e-16
    assert abs(got[137 * N + 13] - exp[137 * N + 13]) <= 2e-16 * abs(exp[137 * N + 13])
