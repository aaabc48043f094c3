"""GPU tests of the on-device SVQB (skinny_svqb) against the CPU restatement of svqb/svqb.cu:72-130.

Bars: the orthogonalised Q matches the oracle's Q column by column (eigenvectors compared up to
sign) within 1e-9 relative for moderately conditioned inputs; the device-reported ||Q^T Q - I||_F
equals the oracle's measurement of the same Q; two passes reach 1e-13.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

from oracle import svqb as OS  # noqa: E402


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def align_signs(Q, Qr, K, M):
    Q2, R2 = Q.reshape(K, M), Qr.reshape(K, M)
    s = np.sign(np.sum(Q2 * R2, axis=0))
    return (Q2 * s[None, :]).ravel()


@pytest.mark.parametrize("M", [1, 4, 16, 33, 64])
@pytest.mark.parametrize("gram", ["native", "dd", "split"])
def test_svqb_matches_oracle(handle, M, gram):
    K = 20000
    X = OS.make_x(K, M, 1e3, seed=M)
    Xd = dev(X)
    err = handle.svqb(K, M, Xd, M, gram_acc=gram)
    torch.cuda.synchronize()
    Q = Xd.cpu().numpy()
    Qr = OS.svqb(X, K, M, "exact")
    Qa = align_signs(Q, Qr, K, M)
    rel = np.linalg.norm(Qa - Qr) / np.linalg.norm(Qr)
    assert rel <= 1e-9, rel
    ref_err = OS.orth_error(Q, K, M)
    assert abs(err - ref_err) <= 1e-12 + 1e-6 * ref_err, (err, ref_err)
    assert err <= 1e-10


def test_svqb_two_passes_ill_conditioned(handle):
    """cond(X) = 1e8 (the precision workload's range): one pass leaves ~kappa^2 u, a second pass
    restores orthogonality to working precision."""
    K, M = 1 << 16, 16
    X = OS.make_x(K, M, 1e8, seed=7)
    errs = {}
    for gram in ("native", "dd", "split"):
        Xd = dev(X)
        e1 = handle.svqb(K, M, Xd, M, gram_acc=gram)
        e2 = handle.svqb(K, M, Xd, M, gram_acc=gram)
        errs[gram] = (e1, e2)
        assert np.isfinite(e1) and e2 <= 1e-13, (gram, e1, e2)
    # one pass leaves O(kappa^2 u) whichever Gram is used (the oracle shows 0.08-0.4 here): the
    # loss comes from forming Q, not from the Gram, so no ordering between methods is asserted


def test_svqb_bad_arguments(handle):
    from skinny_matmul_gb300 import SkinnyError
    X = dev(np.zeros(100))
    with pytest.raises(SkinnyError, match="BAD_ARG"):
        handle.svqb(10, 8, X, 4)
    with pytest.raises(SkinnyError, match="UNSUPPORTED"):
        handle.svqb(1, 65, dev(np.zeros(65)), 65)


@pytest.mark.parametrize("M", [1, 5, 16, 40, 64])
@pytest.mark.parametrize("gram", ["native", "split"])
def test_complex_svqb_matches_oracle(handle, M, gram):
    """Complex SVQB (Hermitian Gram, Hermitian Jacobi on the device) against the host oracle
    (LAPACK eigensolver, the same phase convention)."""
    K = 20000
    X = OS.make_x_complex(K, M, 1e3, seed=M)
    Xd = dev(X)
    err = handle.svqb(K, M, Xd, M, gram_acc=gram)
    torch.cuda.synchronize()
    Q = Xd.cpu().numpy()
    Qr = OS.svqb_complex(X, K, M)
    rel = np.linalg.norm(Q - Qr) / np.linalg.norm(Qr)
    assert rel <= 1e-9, rel
    ref_err = OS.orth_error_complex(Q, K, M)
    assert abs(err - ref_err) <= 1e-12 + 1e-6 * ref_err, (err, ref_err)
    assert err <= 1e-10
