"""CPU restatement of the reference's SVQB (svqb/svqb.cu:72-130) and its error metrics.

TEST INFRASTRUCTURE ONLY (imported by tests/ and bench.py's CPU baseline, never by the product).

The reference runs the symmetric eigensolve on the host with MAGMA's dsyevd (svqb.cu:113); MAGMA
is not available here, so numpy.linalg.eigh -- LAPACK dsyevd, the same algorithm family -- stands
in.  The reference pins no eigensolve results, so eigenvector parity is judged up to column signs
(an eigenvector is defined only up to sign) and through ||Q^T Q - I||_F.
"""
from __future__ import annotations

import numpy as np

from . import oracle as O


def make_x(K: int, M: int, cond: float, seed: int) -> np.ndarray:
    """X = G R: G seeded standard Gaussian (K x M), R upper triangular (M x M) with singular values
    log-spaced from 1 to 1/cond (R is the triangular factor of U diag(sigma) V^T for seeded
    orthogonal U, V).  Returns X as a flat row-major array (K x M)."""
    rng = np.random.default_rng(seed)
    G = rng.standard_normal((K, M))
    U, _ = np.linalg.qr(rng.standard_normal((M, M)))
    V, _ = np.linalg.qr(rng.standard_normal((M, M)))
    sig = np.logspace(0, -np.log10(cond), M)
    _, R = np.linalg.qr(U @ np.diag(sig) @ V.T)
    return np.ascontiguousarray((G @ R).ravel())


def gram(X: np.ndarray, K: int, M: int, method: str = "exact") -> np.ndarray:
    """S = X^T X as an (M x M) array; 'exact' rounds the exact sum once, 'plain' uses FP64 loops."""
    if method == "exact":
        hi, lo = O.tsmttsm_exact(M, M, K, X, M, X, M)
        return (hi + lo).reshape(M, M).T
    S = np.zeros(M * M)
    O.tsmttsm(M, M, K, X, M, 1.0, X, M, 0.0, S, M)
    return S.reshape(M, M).T


def svqb_transform(S: np.ndarray) -> np.ndarray:
    """T = D U diag(1/sqrt(max(1e-15, lambda))) as in svqb.cu:99-119 (eigenvalues ascending),
    returned as an M x M array with X_new = X @ T."""
    M = S.shape[0]
    diag = np.diag(S)
    d = np.where(np.abs(diag) > 1.0e-15, 1.0 / np.sqrt(np.abs(diag)), 0.0)
    Ss = S * d[:, None] * d[None, :]
    lam, U = np.linalg.eigh(Ss)
    # sign convention shared with the device solver: largest-magnitude entry positive
    idx = np.argmax(np.abs(U), axis=0)
    U = U * np.sign(U[idx, np.arange(M)])[None, :]
    return U * d[:, None] / np.sqrt(np.maximum(1.0e-15, lam))[None, :]


def svqb(X: np.ndarray, K: int, M: int, method: str = "exact") -> np.ndarray:
    """One SVQB pass; returns Q (flat, K x M)."""
    T = svqb_transform(gram(X, K, M, method))
    return (X.reshape(K, M) @ T).ravel()


def orth_error(Q: np.ndarray, K: int, M: int) -> float:
    """||Q^T Q - I||_F with the Gram formed exactly (svqb.cu:184-211 uses a double-double Gram)."""
    S = gram(Q, K, M, "exact")
    return float(np.linalg.norm(S - np.eye(M)))


def make_x_complex(K: int, M: int, cond: float, seed: int = 0) -> np.ndarray:
    """Complex X = G R: G complex Gaussian K x M, R upper triangular with singular values
    log-spaced from 1 to 1/cond (as make_x, complex)."""
    rng = np.random.default_rng(seed)
    U, _ = np.linalg.qr(rng.standard_normal((M, M)) + 1j * rng.standard_normal((M, M)))
    V, _ = np.linalg.qr(rng.standard_normal((M, M)) + 1j * rng.standard_normal((M, M)))
    sig = np.logspace(0, -np.log10(cond), M)
    _, R = np.linalg.qr(U @ np.diag(sig) @ V.conj().T)
    G = rng.standard_normal((K, M)) + 1j * rng.standard_normal((K, M))
    return np.ascontiguousarray(G @ R).ravel()


def svqb_complex(X: np.ndarray, K: int, M: int) -> np.ndarray:
    """Host SVQB of a complex block with the Hermitian Gram (test oracle of skinny_svqb_z):
    S = X^H X, D^-1/2 scaling, eigendecomposition (LAPACK), eigenvalues ascending, each
    eigenvector's largest-magnitude entry real positive, Q = X D U Lambda^-1/2."""
    Xm = X.reshape(K, M)
    S = Xm.conj().T @ Xm
    sd = np.real(np.diag(S))
    d = np.where(np.abs(sd) > 1e-15, 1.0 / np.sqrt(np.abs(sd)), 0.0)
    w, U = np.linalg.eigh(S * d[:, None] * d[None, :])
    for c in range(M):
        k = int(np.argmax(np.abs(U[:, c])))
        U[:, c] *= np.conj(U[k, c]) / abs(U[k, c])
    T = (d[:, None] * U) / np.sqrt(np.maximum(1e-15, w))[None, :]
    return (Xm @ T).ravel()


def orth_error_complex(Q: np.ndarray, K: int, M: int) -> float:
    Qm = Q.reshape(K, M)
    return float(np.linalg.norm(Qm.conj().T @ Qm - np.eye(M)))
