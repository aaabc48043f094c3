"""GPU tests of CholQR / CholQR2 (skinny_cholqr): Gram, on-device Cholesky, in-place TSMM with R^-1.

Bars: CholQR2 orthogonalises to ||Q^T Q - I||_F <= 1e-13 and its Q equals the Q of a Householder
QR (numpy, diagonal of R made positive) within 1e-10 for condition numbers up to 1e5; the device's
orthogonality figure equals the host's measurement; a Gram that is not positive definite is an
error, not a silent result."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

from oracle import svqb as OS  # noqa: E402


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("M", [1, 3, 16, 33, 64])
@pytest.mark.parametrize("gram", ["native", "split", "dd"])
def test_cholqr2_matches_householder_qr(handle, M, gram):
    K = 30000
    X = OS.make_x(K, M, 1e5, seed=M + 1)
    Xd = dev(X)
    err = handle.cholqr(K, M, Xd, M, passes=2, gram_acc=gram)
    Q = Xd.cpu().numpy().reshape(K, M)
    Qh, R = np.linalg.qr(X.reshape(K, M))
    Qh = Qh * np.sign(np.diag(R))[None, :]
    assert np.linalg.norm(Q - Qh) / np.linalg.norm(Qh) <= 1e-10
    ref = OS.orth_error(Q.ravel(), K, M)
    assert abs(err - ref) <= 1e-12 + 1e-6 * ref
    assert err <= 1e-13


def test_cholqr_one_pass_loses_as_kappa_squared(handle):
    K, M = 1 << 16, 16
    X = OS.make_x(K, M, 1e6, seed=3)
    e1 = handle.cholqr(K, M, dev(X), M, passes=1, gram_acc="split")
    e2 = handle.cholqr(K, M, dev(X), M, passes=2, gram_acc="split")
    assert 1e-8 < e1 < 10 and e2 <= 1e-13, (e1, e2)


def test_cholqr_padded_rows_and_not_positive_definite(handle):
    from skinny_matmul_gb300 import lib as L
    rng = np.random.default_rng(4)
    K, M, ldx = 5000, 7, 9
    X = rng.standard_normal(K * ldx)
    Xd = dev(X)
    err = handle.cholqr(K, M, Xd, ldx, passes=2)
    Q = Xd.cpu().numpy().reshape(K, ldx)
    assert np.array_equal(Q[:, M:], X.reshape(K, ldx)[:, M:])  # padding untouched
    assert err <= 1e-13
    Z = rng.standard_normal((K, M))
    Z[:, 4] = 0.0
    with pytest.raises(L.SkinnyError):
        handle.cholqr(K, M, dev(Z.ravel()), M, passes=1)
