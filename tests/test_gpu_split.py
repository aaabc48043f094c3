"""GPU parity tests of the FP64 split-precision TSMTTSM (tcgen05 tensor cores) against the oracle.

Bars: golden integer cases bit-exact; random data within the FP64 bound 8 sqrt(K) 2^-53 normwise
against the exact oracle and, for the wide-exponent workload (s * 2^e, e in [-20, 20]), within
1e-15 normwise; results independent of the launch (deterministic).
"""
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


SPLIT_CASES = [c for c in common.int_cases() if c["op"] == "tsmttsm" and not c["cplx"] and c["M"] <= 128 and
               c["N"] <= 128]


@pytest.mark.parametrize("case", SPLIT_CASES, ids=lambda c: c["id"])
def test_split_golden_integer_cases_bit_exact(handle, case):
    c = case
    A, B, C = dev(c["A"]), dev(c["B"]), dev(c["C"])
    if c["self"]:
        B = A
    handle.tsmttsm(c["M"], c["N"], c["K"], A, c["lda"], 1.0, B, c["ldb"], float(c["beta"]), C, c["ldc"], acc="split")
    assert np.array_equal(host(C), c["exp"])


FP32_CASES = [c for c in common.int_cases() if c["op"] == "tsmttsm" and c["M"] <= (64 if c["cplx"] else 128) and
              c["N"] <= (64 if c["cplx"] else 128)]


@pytest.mark.parametrize("case", FP32_CASES, ids=lambda c: c["id"])
def test_split_fp32_golden_integer_cases_bit_exact(handle, case):
    """The integer fixtures in FP32 / complex FP32 storage (exact in both) on the split kernel."""
    c = case
    dt = np.complex64 if c["cplx"] else np.float32
    A, B, C = dev(c["A"].astype(dt)), dev(c["B"].astype(dt)), dev(c["C"].astype(dt))
    if c["self"]:
        B = A
    handle.tsmttsm(c["M"], c["N"], c["K"], A, c["lda"], 1.0, B, c["ldb"], float(c["beta"]), C, c["ldc"], acc="split")
    assert np.array_equal(host(C).astype(np.complex128 if c["cplx"] else np.float64), c["exp"])


@pytest.mark.parametrize("dt", [np.float32, np.complex64])
@pytest.mark.parametrize("M,N,K", [(1, 1, 1000), (4, 4, 33333), (8, 8, 1 << 18), (16, 16, 50000), (3, 7, 4097),
                                   (8, 2, 129), (32, 32, 20000), (64, 64, 9000), (20, 41, 3001), (128, 16, 2000),
                                   (24, 19, 5001)])
def test_split_fp32_vs_exact(handle, dt, M, N, K):
    """FP32 / complex FP32 storage on the split kernels (exact products, FP64-accurate sums, one
    rounding to FP32): within 2^-23 normwise of the exact result, where FP32 accumulation is held
    to 8 sqrt(K) 2^-24.  Widths above 16 take the wide kernel (odd widths its element-wise copy
    path); complex widths up to 64 (their real product is 128 wide)."""
    cplx = dt == np.complex64
    if cplx and max(M, N) > 64:
        pytest.skip("complex split TSMTTSM: M, N <= 64")
    rng = np.random.default_rng(M * 31 + N * 7 + K + 5)
    lda, ldb, ldc = M, N, M + 2
    A = common.uniform(rng, K * lda, dt)
    B = common.uniform(rng, K * ldb, dt)
    C0 = common.uniform(rng, N * ldc, dt)
    alpha, beta = (1.25 + 0.5j, -0.5 + 0.25j) if cplx else (1.25, -0.5)
    Cd = dev(C0)
    handle.tsmttsm(M, N, K, dev(A), lda, alpha, dev(B), ldb, beta, Cd, ldc, acc="split")
    got = host(Cd)
    exp, den = common.tsmttsm_expected(M, N, K, A, lda, B, ldb, C0, ldc, alpha, beta)
    err = common.normwise(got, exp, den, common.c_mask_tsmttsm(M, N, ldc))
    assert err <= 2.0 ** -23, err


def test_split_fp32_gram_and_beyond_the_limit(handle):
    """FP32 Gram (A == B, mirrored 64 x 64 blocks) within the bound; widths above 128 refused."""
    from skinny_matmul_gb300 import SkinnyError
    rng = np.random.default_rng(77)
    M, K = 96, 5000
    A = common.uniform(rng, K * M, np.float32)
    Ad, Cd = dev(A), dev(np.zeros(M * M, np.float32))
    handle.tsmttsm(M, M, K, Ad, M, 1.0, Ad, M, 0.0, Cd, M, acc="split")
    exp, den = common.tsmttsm_expected(M, M, K, A, M, A, M, np.zeros(M * M, np.float32), M, 1.0, 0.0)
    assert common.normwise(host(Cd), exp, den) <= 2.0 ** -23
    X = dev(np.zeros(130 * 64, np.float32))
    C = dev(np.zeros(130 * 130, np.float32))
    with pytest.raises(SkinnyError, match="UNSUPPORTED"):
        handle.tsmttsm(130, 130, 64, X, 130, 1.0, X[1:], 130, 0.0, C, 130, acc="split")


SHAPES = [(1, 1, 1000), (2, 2, 70000), (4, 4, 33333), (8, 8, 1 << 20), (16, 16, 100000), (4, 16, 12345),
          (16, 4, 12345), (5, 3, 1001), (13, 7, 4096), (8, 8, 127), (8, 8, 129), (3, 3, 1)]


@pytest.mark.parametrize("M,N,K", SHAPES)
def test_split_uniform_vs_exact(handle, M, N, K):
    rng = np.random.default_rng(M * 31 + N * 7 + K)
    lda, ldb, ldc = M, N, M + 2
    A = rng.uniform(-1, 1, K * lda)
    B = rng.uniform(-1, 1, K * ldb)
    C0 = rng.uniform(-1, 1, N * ldc)
    Cd = dev(C0)
    handle.tsmttsm(M, N, K, dev(A), lda, 1.25, dev(B), ldb, -0.5, Cd, ldc, acc="split")
    got = host(Cd)
    exp, den = common.tsmttsm_expected(M, N, K, A, lda, B, ldb, C0, ldc, 1.25, -0.5)
    err = common.normwise(got, exp, den, common.c_mask_tsmttsm(M, N, ldc))
    assert err <= common.tol(np.float64, K), err
    assert err <= 4e-16, err  # the split sum is formed exactly per period; only FP64 window sums round


@pytest.mark.parametrize("M", [8, 16])
def test_split_wide_exponents_c3_distribution(handle, M):
    """Entries s * 2^e, s in U[1,2), random sign, e in [-20, 20] (the precision workload)."""
    rng = np.random.default_rng(100 + M)
    K = 1 << 17
    A = common.spread(rng, K * M)
    B = common.spread(rng, K * M)
    Cd = dev(np.zeros(M * M))
    handle.tsmttsm(M, M, K, dev(A), M, 1.0, dev(B), M, 0.0, Cd, M, acc="split")
    got = host(Cd)
    exp, den = common.tsmttsm_expected(M, M, K, A, M, B, M, np.zeros(M * M), M, 1.0, 0.0)
    err = common.normwise(got, exp, den)
    assert err <= 1e-15, err
    # the CUDA-core FP64 result for comparison: the split result is at least as accurate
    Cp = dev(np.zeros(M * M))
    handle.tsmttsm(M, M, K, dev(A), M, 1.0, dev(B), M, 0.0, Cp, M, acc="native")
    assert err <= 2 * common.normwise(host(Cp), exp, den) + 1e-17


def test_split_gram_and_growing_exponents(handle):
    """Gram mode, with row magnitudes growing along K so column exponents rise mid-stream and
    force new accumulation periods."""
    rng = np.random.default_rng(5)
    M, K = 12, 200003
    scale = np.ldexp(1.0, (np.arange(K) // 5000) - 20)
    X = (rng.uniform(-1, 1, (K, M)) * scale[:, None]).ravel()
    Sd = dev(np.zeros(M * M))
    Xd = dev(X)
    handle.tsmttsm(M, M, K, Xd, M, 1.0, Xd, M, 0.0, Sd, M, acc="split")
    got = host(Sd)
    exp, den = common.tsmttsm_expected(M, M, K, X, M, X, M, np.zeros(M * M), M, 1.0, 0.0)
    assert common.normwise(got, exp, den) <= 4e-16


def test_split_unaligned_padded_and_zero_columns(handle):
    rng = np.random.default_rng(8)
    M, N, K = 8, 6, 50001
    lda, ldb = M + 3, N + 1
    A = rng.uniform(-1, 1, K * lda + 1)
    B = rng.uniform(-1, 1, K * ldb + 1)
    A.reshape(-1)[1:][: K * lda].reshape(K, lda)[:, 2] = 0.0  # an all-zero column
    Ad, Bd = dev(A), dev(B)
    for off in (0, 1):
        Cd = dev(np.zeros(N * M))
        handle.tsmttsm(M, N, K, Ad[off:], lda, 1.0, Bd[off:], ldb, 0.0, Cd, M, acc="split")
        exp, den = common.tsmttsm_expected(M, N, K, A[off:].copy(), lda, B[off:].copy(), ldb, np.zeros(M * N), M,
                                           1.0, 0.0)
        assert common.normwise(host(Cd), exp, den) <= 4e-16, off


def test_split_deterministic_and_auto(handle):
    rng = np.random.default_rng(2)
    M = N = 16  # auto picks the split kernel from M * N >= 256 on
    K = 1 << 20
    A, B = dev(rng.uniform(-1, 1, K * M)), dev(rng.uniform(-1, 1, K * N))
    outs = []
    for acc in ("split", "split", "auto"):
        Cd = dev(np.zeros(M * N))
        handle.tsmttsm(M, N, K, A, M, 1.0, B, N, 0.0, Cd, M, acc=acc)
        outs.append(host(Cd))
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[0], outs[2])
    handle.check_device()


# M or N > 16: the wide kernel (64 x 64 blocks of C in one launch, each element sliced once per
# block row / column; Gram computes the upper blocks only and mirrors them)
BLOCKED = [(32, 32, 20011), (64, 64, 8192), (128, 128, 4099), (17, 40, 7000), (64, 20, 9000), (20, 64, 9000),
           (128, 16, 3000), (1, 128, 3000), (33, 33, 129), (65, 63, 5000), (96, 128, 2000), (128, 1, 999)]


@pytest.mark.parametrize("M,N,K", BLOCKED)
@pytest.mark.parametrize("pad", [0, 1, 2])
def test_split_blocked_vs_exact(handle, M, N, K, pad):
    """pad 0: dense rows (whole stages by one copy); 1: odd leading dimension (8-byte copies);
    2: even padded rows (one bulk copy per row)."""
    rng = np.random.default_rng(M * 131 + N * 7 + K + pad)
    lda, ldb, ldc = M + pad, N + pad, M + 3
    A = rng.uniform(-1, 1, K * lda)
    B = rng.uniform(-1, 1, K * ldb)
    C0 = rng.uniform(-1, 1, N * ldc)
    Cd = dev(C0)
    handle.tsmttsm(M, N, K, dev(A), lda, 0.75, dev(B), ldb, 1.5, Cd, ldc, acc="split")
    got = host(Cd)
    exp, den = common.tsmttsm_expected(M, N, K, A, lda, B, ldb, C0, ldc, 0.75, 1.5)
    err = common.normwise(got, exp, den, common.c_mask_tsmttsm(M, N, ldc))
    assert err <= 4e-16, err
    assert np.array_equal(got[~common.c_mask_tsmttsm(M, N, ldc)], C0[~common.c_mask_tsmttsm(M, N, ldc)])


# M, N <= 32 with one of them > 16: the wide kernel's folded stages (32 rows per stage; rows
# 16..31 fill the second half of the 64-row digit planes, the two diagonal quadrants are added)
FOLDED = [(17, 17, 1001), (32, 8, 40001), (24, 31, 4097), (20, 1, 3000), (32, 32, 65), (29, 18, 33),
          (1, 32, 777)]


@pytest.mark.parametrize("M,N,K", FOLDED)
@pytest.mark.parametrize("pad", [0, 1, 2])
def test_split_folded_vs_exact(handle, M, N, K, pad):
    """The same bars as the blocked shapes, for every copy path (dense, 8-byte, per-row bulk)."""
    rng = np.random.default_rng(M * 17 + N * 5 + K + pad)
    lda, ldb, ldc = M + pad, N + pad, M + 1
    A = rng.uniform(-1, 1, K * lda)
    B = rng.uniform(-1, 1, K * ldb)
    C0 = rng.uniform(-1, 1, N * ldc)
    Cd = dev(C0)
    handle.tsmttsm(M, N, K, dev(A), lda, -1.25, dev(B), ldb, 0.5, Cd, ldc, acc="split")
    got = host(Cd)
    exp, den = common.tsmttsm_expected(M, N, K, A, lda, B, ldb, C0, ldc, -1.25, 0.5)
    mask = common.c_mask_tsmttsm(M, N, ldc)
    assert common.normwise(got, exp, den, mask) <= 4e-16
    assert np.array_equal(got[~mask], C0[~mask])


@pytest.mark.parametrize("K", [1, 15, 16, 17, 31, 32, 33, 255, 256, 257, 4095, 4097])
def test_split_folded_small_k(handle, K):
    rng = np.random.default_rng(K + 3)
    M, N = 32, 20
    A, B = rng.uniform(-1, 1, K * M), rng.uniform(-1, 1, K * N)
    C0 = rng.uniform(-1, 1, M * N)
    Cd = dev(C0)
    handle.tsmttsm(M, N, K, dev(A), M, 2.0, dev(B), N, 0.5, Cd, M, acc="split")
    exp, den = common.tsmttsm_expected(M, N, K, A, M, B, N, C0, M, 2.0, 0.5)
    assert common.normwise(host(Cd), exp, den) <= 4e-16


def test_split_folded_row_halves_with_different_exponents(handle):
    """Rows 16..31 of every 32-row stage are 2^12 larger than rows 0..15, and the scale grows
    along K: the two plane halves of a column carry different exponents and start new epochs at
    different stages.  Gram of the same data is mirrored and deterministic."""
    rng = np.random.default_rng(5)
    M, N, K = 24, 32, 90001
    k = np.arange(K)
    scale = np.ldexp(1.0, 12 * ((k // 16) % 2) + (k // 9000) - 5)
    A = (rng.uniform(-1, 1, (K, M)) * scale[:, None])
    B = rng.uniform(-1, 1, (K, N))
    A[:, 3] = 0.0
    B[: K // 3, 30] = 0.0
    A, B = A.ravel(), B.ravel()
    Cd = dev(np.zeros(M * N))
    handle.tsmttsm(M, N, K, dev(A), M, 1.0, dev(B), N, 0.0, Cd, M, acc="split")
    exp, den = common.tsmttsm_expected(M, N, K, A, M, B, N, np.zeros(M * N), M, 1.0, 0.0)
    assert common.normwise(host(Cd), exp, den) <= 4e-16
    Ad = dev(A)
    outs = []
    for _ in range(2):
        Gd = dev(np.zeros(M * M))
        handle.tsmttsm(M, M, K, Ad, M, 1.0, Ad, M, 0.0, Gd, M, acc="split")
        outs.append(host(Gd))
    assert np.array_equal(outs[0], outs[1])
    G = outs[0].reshape(M, M)
    assert np.array_equal(G, G.T)
    exp, den = common.tsmttsm_expected(M, M, K, A, M, A, M, np.zeros(M * M), M, 1.0, 0.0)
    assert common.normwise(outs[0], exp, den) <= 4e-16


@pytest.mark.parametrize("M", [17, 32, 40, 64, 128])
@pytest.mark.parametrize("beta", [0.0, -0.5])
def test_split_blocked_gram_mirrored(handle, M, beta):
    rng = np.random.default_rng(M + 7)
    K = 6000 if M == 128 else 30000
    X = common.spread(rng, K * M)
    C0 = rng.uniform(-1, 1, M * M)
    Cd = dev(C0)
    Xd = dev(X)
    handle.tsmttsm(M, M, K, Xd, M, 1.0, Xd, M, beta, Cd, M, acc="split")
    got = host(Cd)
    exp, den = common.tsmttsm_expected(M, M, K, X, M, X, M, C0, M, 1.0, beta)
    assert common.normwise(got, exp, den) <= 1e-15
    if beta == 0.0:
        G = got.reshape(M, M)
        assert np.array_equal(G, G.T)


def test_split_blocked_wide_exponents_and_determinism(handle):
    rng = np.random.default_rng(9)
    M = N = 64
    K = 1 << 16
    A, B = common.spread(rng, K * M), common.spread(rng, K * N)
    Ad, Bd = dev(A), dev(B)
    outs = []
    for _ in range(2):
        Cd = dev(np.zeros(M * N))
        handle.tsmttsm(M, N, K, Ad, M, 1.0, Bd, N, 0.0, Cd, M, acc="split")
        outs.append(host(Cd))
    assert np.array_equal(outs[0], outs[1])
    exp, den = common.tsmttsm_expected(M, N, K, A, M, B, N, np.zeros(M * N), M, 1.0, 0.0)
    assert common.normwise(outs[0], exp, den) <= 1e-15


def test_split_beyond_128_unsupported_and_auto_falls_back(handle):
    from skinny_matmul_gb300 import lib as L
    M, N, K = 136, 8, 4096
    rng = np.random.default_rng(1)
    A, B = dev(rng.uniform(-1, 1, K * M)), dev(rng.uniform(-1, 1, K * N))
    Cd = dev(np.zeros(M * N))
    with pytest.raises(L.SkinnyError):
        handle.tsmttsm(M, N, K, A, M, 1.0, B, N, 0.0, Cd, M, acc="split")
    handle.tsmttsm(M, N, K, A, M, 1.0, B, N, 0.0, Cd, M, acc="auto")  # native FP64
    exp, den = common.tsmttsm_expected(M, N, K, host(A), M, host(B), N, np.zeros(M * N), M, 1.0, 0.0)
    assert common.normwise(host(Cd), exp, den) <= common.tol(np.float64, K)


def test_split_wide_growing_exponents_and_zero_columns(handle):
    """Column maxima rise along K (new exponent epochs mid-stream), some columns are zero, others
    are zero until late."""
    rng = np.random.default_rng(21)
    M, N, K = 64, 48, 150001
    scale = np.ldexp(1.0, (np.arange(K) // 7000) - 10)
    A = (rng.uniform(-1, 1, (K, M)) * scale[:, None])
    B = rng.uniform(-1, 1, (K, N))
    A[:, 5] = 0.0
    B[:, 7] = 0.0
    A[: K // 2, 9] = 0.0
    B[: K - 100, 11] = 0.0
    A, B = A.ravel(), B.ravel()
    Cd = dev(np.zeros(M * N))
    handle.tsmttsm(M, N, K, dev(A), M, 1.0, dev(B), N, 0.0, Cd, M, acc="split")
    exp, den = common.tsmttsm_expected(M, N, K, A, M, B, N, np.zeros(M * N), M, 1.0, 0.0)
    assert common.normwise(host(Cd), exp, den) <= 4e-16


@pytest.mark.parametrize("M,N,lda,ldb,off", [(33, 31, 33, 31, 0), (40, 40, 41, 43, 0), (64, 64, 64, 64, 1),
                                              (17, 64, 20, 70, 1)])
def test_split_wide_unaligned_and_odd(handle, M, N, lda, ldb, off):
    rng = np.random.default_rng(M + N + lda)
    K = 20000
    A = rng.uniform(-1, 1, K * lda + 1)
    B = rng.uniform(-1, 1, K * ldb + 1)
    Ad, Bd = dev(A), dev(B)
    Cd = dev(np.zeros(N * M))
    handle.tsmttsm(M, N, K, Ad[off:], lda, 1.0, Bd[off:], ldb, 0.0, Cd, M, acc="split")
    exp, den = common.tsmttsm_expected(M, N, K, A[off:].copy(), lda, B[off:].copy(), ldb, np.zeros(M * N), M, 1.0,
                                       0.0)
    assert common.normwise(host(Cd), exp, den) <= 4e-16


@pytest.mark.parametrize("K", [1, 15, 16, 17, 127, 128, 129, 2047, 2048, 2049])
def test_split_wide_small_k(handle, K):
    rng = np.random.default_rng(K)
    M, N = 48, 64
    A, B = rng.uniform(-1, 1, K * M), rng.uniform(-1, 1, K * N)
    C0 = rng.uniform(-1, 1, M * N)
    Cd = dev(C0)
    handle.tsmttsm(M, N, K, dev(A), M, 2.0, dev(B), N, 0.5, Cd, M, acc="split")
    exp, den = common.tsmttsm_expected(M, N, K, A, M, B, N, C0, M, 2.0, 0.5)
    assert common.normwise(host(Cd), exp, den) <= 4e-16
