"""GPU parity tests of the complex FP64 TSMTTSM in split precision (the real product of doubled
width on the split kernels, then one combination kernel) against the oracle.

Bars: golden integer cases bit-exact; random data within min(8 sqrt(K) u, 8e-16) normwise of the
exact oracle (u = 2^-53)."""
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


CASES = [c for c in common.int_cases() if c["op"] == "tsmttsm" and c["cplx"]]


@pytest.mark.parametrize("case", CASES, ids=lambda c: c["id"])
def test_split_complex_golden_bit_exact(handle, case):
    c = case
    A, B, C = dev(c["A"]), dev(c["B"]), dev(c["C"])
    if c["self"]:
        B = A
    handle.tsmttsm(c["M"], c["N"], c["K"], A, c["lda"], 1.0, B, c["ldb"], complex(c["beta"]), C, c["ldc"],
                   acc="split")
    assert np.array_equal(host(C), c["exp"])


SHAPES = [(1, 1, 5000), (4, 4, 20000), (8, 8, 30011), (3, 5, 7777), (16, 16, 20000), (32, 32, 12345),
          (64, 64, 6000), (17, 40, 5000), (64, 1, 3000), (9, 8, 129)]


@pytest.mark.parametrize("M,N,K", SHAPES)
def test_split_complex_uniform(handle, M, N, K):
    rng = np.random.default_rng(M * 37 + N + K)
    lda, ldb, ldc = M, N + 1, M + 2
    A = common.uniform(rng, K * lda, np.complex128)
    B = common.uniform(rng, K * ldb, np.complex128)
    C0 = common.uniform(rng, N * ldc, np.complex128)
    alpha, beta = 0.75 - 0.5j, 0.25 + 1.0j
    Cd = dev(C0)
    handle.tsmttsm(M, N, K, dev(A), lda, alpha, dev(B), ldb, beta, Cd, ldc, acc="split")
    got = host(Cd)
    exp, den = common.tsmttsm_expected(M, N, K, A, lda, B, ldb, C0, ldc, alpha, beta)
    err = common.normwise(got, exp, den, common.c_mask_tsmttsm(M, N, ldc))
    assert err <= min(common.tol(np.complex128, K), 8e-16), err


@pytest.mark.parametrize("M", [4, 24, 64])
def test_split_complex_gram_and_auto(handle, M):
    rng = np.random.default_rng(M)
    K = 40000
    X = common.uniform(rng, K * M, np.complex128)
    Xd = dev(X)
    out = []
    for acc in ("split", "auto"):
        Cd = dev(np.zeros(M * M, np.complex128))
        handle.tsmttsm(M, M, K, Xd, M, 1.0, Xd, M, 0.0, Cd, M, acc=acc)
        out.append(host(Cd))
    exp, den = common.tsmttsm_expected(M, M, K, X, M, X, M, np.zeros(M * M, np.complex128), M, 1.0, 0.0)
    assert common.normwise(out[0], exp, den) <= 8e-16
    assert common.normwise(out[1], exp, den) <= common.tol(np.complex128, K)


def test_split_complex_too_wide_unsupported(handle):
    from skinny_matmul_gb300 import lib as L
    M, N, K = 65, 2, 1000
    A, B = dev(np.zeros(K * M, np.complex128)), dev(np.zeros(K * N, np.complex128))
    Cd = dev(np.zeros(M * N, np.complex128))
    with pytest.raises(L.SkinnyError):
        handle.tsmttsm(M, N, K, A, M, 1.0, B, N, 0.0, Cd, M, acc="split")


@pytest.mark.parametrize("acc", ["native", "split", "auto"])
@pytest.mark.parametrize("M,N,K", [(1, 1, 3000), (4, 4, 20000), (8, 3, 7001), (16, 16, 9000), (40, 24, 5000),
                                   (64, 64, 4000)])
def test_conjugate_transpose(handle, acc, M, N, K):
    """C = alpha A^H B + beta C (skinny_tsmttsm_conj) against the oracle given conj(A)."""
    rng = np.random.default_rng(M + 3 * N + K)
    A = common.uniform(rng, K * M, np.complex128)
    B = common.uniform(rng, K * N, np.complex128)
    C0 = common.uniform(rng, N * M, np.complex128)
    alpha, beta = 0.5 - 1.0j, -0.25 + 0.5j
    Cd = dev(C0)
    handle.tsmttsm(M, N, K, dev(A), M, alpha, dev(B), N, beta, Cd, M, acc=acc, conj=True)
    exp, den = common.tsmttsm_expected(M, N, K, np.conj(A), M, B, N, C0, M, alpha, beta)
    err = common.normwise(host(Cd), exp, den)
    assert err <= common.tol(np.complex128, K), err
    if acc == "split":
        assert err <= 8e-16


@pytest.mark.parametrize("dt", [np.complex64, np.complex128])
def test_conjugate_gram_is_hermitian_and_real_dtypes_unchanged(handle, dt):
    rng = np.random.default_rng(11)
    M, K = 12, 30000
    X = common.uniform(rng, K * M, dt)
    Xd = dev(X)
    Cd = dev(np.zeros(M * M, dt))
    handle.tsmttsm(M, M, K, Xd, M, 1.0, Xd, M, 0.0, Cd, M, acc="native", conj=True)
    G = host(Cd).reshape(M, M)
    assert np.allclose(G, G.conj().T, rtol=0, atol=1e-4 if dt == np.complex64 else 1e-10)
    assert np.all(np.diag(G).real > 0) and np.max(np.abs(np.diag(G).imag)) <= (1e-2 if dt == np.complex64 else 1e-9)
    R = rng.uniform(-1, 1, K * M)
    Rd = dev(R)
    C1, C2 = dev(np.zeros(M * M)), dev(np.zeros(M * M))
    handle.tsmttsm(M, M, K, Rd, M, 1.0, Rd, M, 0.0, C1, M, acc="native", conj=True)
    handle.tsmttsm(M, M, K, Rd, M, 1.0, Rd, M, 0.0, C2, M, acc="native")
    assert np.array_equal(host(C1), host(C2))
