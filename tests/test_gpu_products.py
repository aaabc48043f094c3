"""GPU parity tests of TSMTTSM / TSMM through the C ABI against the CPU oracle.

Bars (written into each assertion):
  * golden integer cases (test.cu fixture design): bit-exact, every dtype and method;
  * random data: normwise error ||C - C*||_F / || |alpha| |A|^T|B| + |beta| |C0| ||_F <= 8 sqrt(K) u
    (K for TSMTTSM, M for TSMM; u = 2^-24 float, 2^-53 double) against the exact oracle;
  * double-double accumulation: within the output rounding of the exact result (<= 2^-52 normwise
    for FP64, 2^-51 complex FP64, 2^-23 FP32 and complex FP32, whose double-double method is FP64
    accumulation of exact products).
"""
import math

import numpy as np
import pytest

import common

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

TORCH = {np.dtype(np.float32): "float32", np.dtype(np.float64): "float64",
         np.dtype(np.complex64): "complex64", np.dtype(np.complex128): "complex128"}


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


REAL = [(np.float32, "native"), (np.float64, "native"), (np.float64, "dd"), (np.float32, "dd")]
CPLX = [(np.complex64, "native"), (np.complex128, "native"), (np.complex64, "dd"), (np.complex128, "dd")]


def dd_bound(dt):
    """The double-double method rounds once to the storage type at the end: FP32 and complex FP32
    (FP64 accumulation of exact products) within a float's rounding, FP64 within 2^-52, complex
    FP64 within 2^-51 (the complex alpha and beta products add two roundings)."""
    return {np.float32: 2.0 ** -23, np.complex64: 2.0 ** -23, np.float64: 2.0 ** -52, np.complex128: 2.0 ** -51}[dt]


def run(handle, op, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, acc="native", stream=None):
    fn = handle.tsmttsm if op == "tsmttsm" else handle.tsmm
    return fn(M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, acc=acc, stream=stream)


CASES = list(common.int_cases())


@pytest.mark.parametrize("case", CASES, ids=lambda c: c["id"])
def test_golden_integer_cases_bit_exact(handle, case):
    c = case
    for dt, acc in (CPLX if c["cplx"] else REAL):
        A = dev(c["A"].astype(dt))
        B = dev(c["B"].astype(dt))
        C = dev(c["C"].astype(dt))
        if c["self"] and c["op"] == "tsmttsm":
            B = A
        if c["self"] and c["op"] == "tsmm":
            A = C
        run(handle, c["op"], c["M"], c["N"], c["K"], A, c["lda"], 1.0, B, c["ldb"], float(c["beta"]), C,
            c["ldc"], acc=acc)
        got = host(C).astype(np.complex128 if c["cplx"] else np.float64)
        assert np.array_equal(got, c["exp"]), (dt, acc)


@pytest.mark.parametrize("op", ["tsmttsm", "tsmm"])
@pytest.mark.parametrize("dt", ["float32", "float64", "complex64", "complex128", "dd"])
def test_reference_shaped_launchers(op, dt):
    """The MatmulFunctionType entry points on the legacy default stream (versions.hpp:43-45)."""
    from skinny_matmul_gb300 import build, launchers
    build.build()
    fn, name = launchers(op, dt)[0]
    cplx = dt.startswith("complex")
    picked = [c for c in CASES if c["op"] == op and c["cplx"] == cplx][::5]
    npdt = {"float32": np.float32, "float64": np.float64, "dd": np.float64, "complex64": np.complex64,
            "complex128": np.complex128}[dt]
    for c in picked:
        A, B, C = dev(c["A"].astype(npdt)), dev(c["B"].astype(npdt)), dev(c["C"].astype(npdt))
        if c["self"] and op == "tsmttsm":
            B = A
        if c["self"] and op == "tsmm":
            A = C
        torch.cuda.synchronize()
        ok = fn(100, c["M"], c["N"], c["K"], A.data_ptr(), c["lda"], 1.0, B.data_ptr(), c["ldb"], float(c["beta"]),
                C.data_ptr(), c["ldc"])
        assert ok, name
        got = host(C).astype(np.complex128 if cplx else np.float64)
        assert np.array_equal(got, c["exp"]), (name, c["id"])


SHAPES_TSMTTSM = [(1, 1, 777), (2, 2, 5000), (4, 4, 33333), (8, 8, 1 << 16), (16, 16, 20000), (32, 32, 9000),
                  (64, 64, 4000), (4, 16, 12345), (16, 4, 12345), (8, 32, 7777), (5, 3, 1001), (128, 128, 600)]


@pytest.mark.parametrize("M,N,K", SHAPES_TSMTTSM)
@pytest.mark.parametrize("dt,acc", REAL + CPLX, ids=lambda x: str(x))
def test_tsmttsm_random_vs_oracle(handle, M, N, K, dt, acc):
    if acc == "dd" and M * N > 4096:
        K = min(K, 2000)
    rng = np.random.default_rng(M * 1000 + N + K)
    lda, ldb, ldc = M, N, M + 1
    A = common.uniform(rng, K * lda, dt)
    B = common.uniform(rng, K * ldb, dt)
    C0 = common.uniform(rng, N * ldc, dt)
    alpha, beta = 1.5, -0.5
    Cd = dev(C0)
    run(handle, "tsmttsm", M, N, K, dev(A), lda, alpha, dev(B), ldb, beta, Cd, ldc, acc=acc)
    got = host(Cd)
    exp, den = common.tsmttsm_expected(M, N, K, A, lda, B, ldb, C0, ldc, alpha, beta)
    err = common.normwise(got, exp, den, common.c_mask_tsmttsm(M, N, ldc))
    bound = dd_bound(dt) if acc == "dd" else common.tol(dt, K)
    assert err <= bound, (err, bound)
    # padding between columns of C untouched
    mask = ~common.c_mask_tsmttsm(M, N, ldc)
    assert np.array_equal(got[mask], C0[mask])


SHAPES_TSMM = [(1, 1), (2, 2), (4, 4), (8, 8), (16, 16), (32, 32), (64, 64), (4, 16), (16, 4), (8, 32), (3, 5)]


@pytest.mark.parametrize("M,N", SHAPES_TSMM)
@pytest.mark.parametrize("dt,acc", REAL + CPLX, ids=lambda x: str(x))
@pytest.mark.parametrize("inplace", [False, True])
def test_tsmm_random_vs_oracle(handle, M, N, dt, acc, inplace):
    if inplace and M != N:
        pytest.skip("in-place covered separately for M != N")
    rng = np.random.default_rng(M * 100 + N)
    K = 20011
    lda, ldb, ldc = M, M + 2, N
    if inplace:
        lda = ldc = max(M, N)
    A = common.uniform(rng, K * lda, dt)
    B = common.uniform(rng, N * ldb, dt)
    C0 = A.copy() if inplace else common.uniform(rng, K * ldc, dt)
    alpha, beta = 1.0, 0.5
    Cd = dev(C0)
    Ad = Cd if inplace else dev(A)
    run(handle, "tsmm", M, N, K, Ad, lda, alpha, dev(B), ldb, beta, Cd, ldc, acc=acc)
    got = host(Cd)
    exp, den = common.tsmm_expected(M, N, K, C0 if inplace else A, lda, B, ldb, C0, ldc, alpha, beta)
    err = common.normwise(got, exp, den, common.c_mask_tsmm(N, K, ldc))
    bound = dd_bound(dt) if acc == "dd" else common.tol(dt, M)
    assert err <= bound, (err, bound)


@pytest.mark.parametrize("M,N", [(4, 8), (8, 4), (3, 16), (16, 1)])
def test_tsmm_inplace_rectangular(handle, M, N):
    rng = np.random.default_rng(M + 10 * N)
    K = 5003
    ld = max(M, N) + 1
    X0 = common.uniform(rng, K * ld, np.float64)
    B = common.uniform(rng, N * M, np.float64)
    Xd = dev(X0)
    handle.tsmm(M, N, K, Xd, ld, 1.0, dev(B), M, 0.25, Xd, ld)
    got = host(Xd)
    exp, den = common.tsmm_expected(M, N, K, X0, ld, B, M, X0, ld, 1.0, 0.25)
    assert common.normwise(got, exp, den, common.c_mask_tsmm(N, K, ld)) <= common.tol(np.float64, M)
    # columns >= N of each row are untouched
    g2, x2 = got.reshape(K, ld), X0.reshape(K, ld)
    assert np.array_equal(g2[:, N:], x2[:, N:])


def test_c1_full_size_tsmttsm(handle):
    """TSMTTSM FP64 8x8, K = 2^20, U[-1,1): the headline TSMTTSM configuration."""
    rng = np.random.default_rng(2024)
    M = N = 8
    K = 1 << 20
    A = rng.uniform(-1, 1, K * M)
    B = rng.uniform(-1, 1, K * N)
    Cd = dev(np.zeros(M * N))
    handle.tsmttsm(M, N, K, dev(A), M, 1.0, dev(B), N, 0.0, Cd, M)
    got = host(Cd)
    exp, den = common.tsmttsm_expected(M, N, K, A, M, B, N, np.zeros(M * N), M, 1.0, 0.0)
    assert common.normwise(got, exp, den) <= common.tol(np.float64, K)


def test_tsmm_full_size_row_sample(handle):
    """TSMM FP64 8x8 with A of 1 GiB (K = 2^24 rows), alpha 1, beta 0.5: checked on sampled rows."""
    M = N = 8
    K = (1 << 30) // (8 * M)
    g = torch.Generator(device="cuda").manual_seed(7)
    A = torch.rand(K * M, dtype=torch.float64, device="cuda", generator=g) * 2 - 1
    C = torch.rand(K * N, dtype=torch.float64, device="cuda", generator=g) * 2 - 1
    B = torch.rand(M * N, dtype=torch.float64, device="cuda", generator=g) * 2 - 1
    rows = torch.randint(0, K, (4096,), device="cuda", generator=g)
    C0 = C.view(K, N)[rows].cpu().numpy()
    A0 = A.view(K, M)[rows].cpu().numpy()
    handle.tsmm(M, N, K, A, M, 1.0, B, M, 0.5, C, N)
    got = C.view(K, N)[rows].cpu().numpy()
    Bm = B.cpu().numpy().reshape(N, M)
    exp = A0 @ Bm.T + 0.5 * C0
    den = np.abs(A0) @ np.abs(Bm).T + 0.5 * np.abs(C0)
    err = np.linalg.norm(got - exp) / np.linalg.norm(den)
    assert err <= common.tol(np.float64, M) + 4 * 2.0 ** -53  # numpy's own reference rounding


def test_kat_on_gpu(handle):
    a, b, d = common.kat()
    N = len(a)
    ex = d["exact_hi"]
    out_dd, out_d = dev(np.zeros(1)), dev(np.zeros(1))
    A, B = dev(a), dev(b)
    handle.tsmttsm(1, 1, N, A, 1, 1.0, B, 1, 0.0, out_dd, 1, acc="dd")
    handle.tsmttsm(1, 1, N, A, 1, 1.0, B, 1, 0.0, out_d, 1, acc="native")
    err_dd = abs(host(out_dd)[0] - ex)
    err_d = abs(host(out_d)[0] - ex)
    assert err_dd < 0.5 * err_d
    assert err_dd / float(np.abs(a) @ np.abs(b)) <= common.tol(np.float64, N)
    a2, b2 = a.copy(), b.copy()
    a2[0] = a2[N - 1] = b2[0] = b2[N - 1] = 0.1
    from oracle import oracle as O
    hi, _ = O.dot_exact(a2, b2)
    out = dev(np.zeros(1))
    handle.tsmttsm(1, 1, N, dev(a2), 1, 1.0, dev(b2), 1, 0.0, out, 1, acc="dd")
    assert abs(host(out)[0] - hi) <= 2 * np.spacing(hi)


@pytest.mark.parametrize("dt", [np.float32, np.complex64, np.complex128])
def test_dd_cancellation(handle, dt):
    """Sums that cancel to 1e-4 of their terms' magnitude.  FP32 and complex FP32: FP64
    accumulation of exact products, so the double-double method returns the exact value rounded
    to the storage type (within one unit), far closer than the native accumulation.  Complex FP64:
    PseudoQuad per component keeps the reference's axpy2, which loses about u |a b| on a cancelling
    step, so its result is held to the normwise bound and to at most the native error."""
    rng = np.random.default_rng(7)
    K = 50000
    a = common.uniform(rng, K, dt)
    b = common.uniform(rng, K, dt)
    cplx = np.iscomplexobj(a)
    # make sum(a * b) small: set the last term so that the float64 sum nearly cancels
    s = np.sum(a[:-1].astype(np.complex128) * b[:-1])
    last = -(s - 1e-4 * (1 + 1j)) / a[-1]
    b[-1] = (last if cplx else last.real).astype(dt)
    exp, den = common.tsmttsm_expected(1, 1, K, a, 1, b, 1, np.zeros(1, dt), 1, 1.0, 0.0)
    out = {}
    for acc in ("dd", "native"):
        o = dev(np.zeros(1, dt))
        handle.tsmttsm(1, 1, K, dev(a), 1, 1.0, dev(b), 1, 0.0, o, 1, acc=acc)
        out[acc] = host(o).astype(np.complex128)[0]
    e = complex(exp[0])
    err_dd, err_n = abs(out["dd"] - e), abs(out["native"] - e)
    if dt in (np.float32, np.complex64):
        ulp = float(np.spacing(np.abs(np.array([e.real, e.imag], dtype=np.float32))).max())
        assert err_dd <= 2 * ulp, (err_dd, ulp)
        assert err_dd < 0.5 * err_n, (err_dd, err_n)
    else:
        assert err_dd / float(den[0]) <= dd_bound(dt), (err_dd, den[0])
        assert err_dd <= err_n, (err_dd, err_n)
    # TSMM 1 x 1 (C = A b over K rows is elementwise) and TSMM with the data as one long row
    M = 64
    A2 = common.uniform(rng, (K // M) * M, dt)
    B2 = common.uniform(rng, M, dt)
    C2 = dev(np.zeros(K // M, dt))
    handle.tsmm(M, 1, K // M, dev(A2), M, 1.0, dev(B2), M, 0.0, C2, 1, acc="dd")
    exp2, den2 = common.tsmm_expected(M, 1, K // M, A2, M, B2, M, np.zeros(K // M, dt), 1, 1.0, 0.0)
    assert common.normwise(host(C2), exp2, den2) <= dd_bound(dt)


def test_edge_k_zero_and_beta_zero_nan(handle):
    M, N = 4, 3
    C0 = np.arange(M * N, dtype=np.float64) + 1
    Cd = dev(C0)
    A = dev(np.zeros(8))
    handle.tsmttsm(M, N, 0, A, M, 2.0, A[1:], N, 0.5, Cd, M)  # K = 0: C = beta * C
    assert np.array_equal(host(Cd), 0.5 * C0)
    # beta == 0 never reads C (NaN must not propagate)
    rng = np.random.default_rng(0)
    K = 1000
    Ah, Bh = rng.uniform(-1, 1, K * M), rng.uniform(-1, 1, K * N)
    Cn = dev(np.full(M * N, np.nan))
    handle.tsmttsm(M, N, K, dev(Ah), M, 1.0, dev(Bh), N, 0.0, Cn, M)
    assert np.isfinite(host(Cn)).all()
    Ct = dev(np.full(K * N, np.nan))
    handle.tsmm(M, N, K, dev(Ah), M, 1.0, dev(rng.uniform(-1, 1, M * N)), M, 0.0, Ct, N)
    assert np.isfinite(host(Ct)).all()


def test_edge_unaligned_and_wide_leading_dims(handle):
    """Operands off a 16-byte boundary and leading dimensions far above the width take the
    plain-load path; results must match the oracle all the same."""
    rng = np.random.default_rng(9)
    M, N, K = 8, 8, 40001
    for lda, ldb, off in ((M, N, 1), (3 * M + 20, N, 0), (M + 1, N + 3, 1)):
        A = rng.uniform(-1, 1, K * lda + 1)
        B = rng.uniform(-1, 1, K * ldb + 1)
        Ad, Bd = dev(A), dev(B)
        Cd = dev(np.zeros(M * N))
        handle.tsmttsm(M, N, K, Ad[off:], lda, 1.0, Bd[off:], ldb, 0.0, Cd, M)
        exp, den = common.tsmttsm_expected(M, N, K, A[off:].copy(), lda, B[off:].copy(), ldb, np.zeros(M * N),
                                           M, 1.0, 0.0)
        assert common.normwise(host(Cd), exp, den) <= common.tol(np.float64, K), (lda, ldb, off)


def test_determinism_and_two_streams(handle):
    rng = np.random.default_rng(4)
    M = N = 8
    K = 300001
    A, B = dev(rng.uniform(-1, 1, K * M)), dev(rng.uniform(-1, 1, K * N))
    C1, C2, C3 = (dev(np.zeros(M * N)) for _ in range(3))
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    torch.cuda.synchronize()
    for _ in range(3):
        handle.tsmttsm(M, N, K, A, M, 1.0, B, N, 0.0, C1, M, stream=s1)
        handle.tsmttsm(M, N, K, A, M, 1.0, B, N, 0.0, C2, M, stream=s2)
    handle.tsmttsm(M, N, K, A, M, 1.0, B, N, 0.0, C3, M)
    assert np.array_equal(host(C1), host(C2)) and np.array_equal(host(C1), host(C3))
    handle.check_device()


def test_bad_arguments(handle):
    from skinny_matmul_gb300 import SkinnyError
    X = dev(np.zeros(64))
    with pytest.raises(SkinnyError, match="BAD_ARG"):
        handle.tsmm(4, 4, 8, X, 4, 1.0, X, 4, 0.0, X, 5)  # in place with lda != ldc
    with pytest.raises(SkinnyError, match="BAD_ARG"):
        handle.tsmttsm(4, 4, 8, X, 4, 1.0, X, 4, 0.0, X, 4)  # C aliases A
    with pytest.raises(SkinnyError, match="BAD_ARG"):
        handle.tsmttsm(4, 4, 8, X, 3, 1.0, X[32:], 4, 0.0, X[16:], 4)  # lda < M
    with pytest.raises(SkinnyError, match="UNSUPPORTED"):  # no double-double conjugate product
        handle.tsmttsm(4, 4, 8, dev(np.zeros(64, np.complex64)), 4, 1.0, dev(np.zeros(64, np.complex64)), 4, 0.0,
                       dev(np.zeros(16, np.complex64)), 4, acc="dd", conj=True)
