"""Parity at the configurations' full sizes, on sampled rows or entries against the exact oracle,
plus size-independent properties where sampling cannot reach (SVQB).

  * C2: TSMM with A of 1 GiB, alpha 1, beta 0.5 -- complex FP64 64 x 64 out of place (real widths
    above 64 run as column / contraction passes), FP64 and complex FP64 64 x 64 in place: 4096
    sampled rows against the exact oracle, 8 sqrt(M) u normwise;
  * C3: FP64 TSMTTSM M = N = 128, K = 2^24, entries s * 2^e (e in [-20, 20]): 8 x 8 sampled entries
    of C (each a length-2^24 dot product) against the exact oracle -- split <= 1e-15 normwise,
    native <= 8 sqrt(K) u, dd <= 2^-52 (output rounding); also the Gram form (A = B);
  * C4: SVQB, K = 2^24, M in {16, 32, 64}, X = G R with condition 1e8: two passes orthogonalise to
    ||Q^T Q - I||_F <= 1e-12 (reported by the device and recomputed independently), Q spans the
    columns of X (||X - Q Q^T X||_F / ||X||_F <= 1e-9), and at condition 1e3 one pass matches the
    host oracle's Q (oracle/svqb.py, FP64 loop Gram).
Inputs are generated on the device from seeded generators (the oracle sees the same values).
"""
import math

import numpy as np
import pytest

import common

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

GIB = 1 << 30


def free():
    torch.cuda.synchronize()
    torch.cuda.empty_cache()


def uniform_dev(n, dtype, g):
    if dtype == torch.complex128:
        return torch.complex(torch.rand(n, dtype=torch.float64, device="cuda", generator=g) * 2 - 1,
                             torch.rand(n, dtype=torch.float64, device="cuda", generator=g) * 2 - 1)
    return torch.rand(n, dtype=dtype, device="cuda", generator=g) * 2 - 1


@pytest.mark.parametrize("dtype,inplace", [(torch.complex128, False), (torch.float64, True),
                                           (torch.complex128, True)], ids=["z-out", "d-in", "z-in"])
def test_c2_tsmm_64x64_full_size_sampled_rows(handle, dtype, inplace):
    M = N = 64
    es = 16 if dtype == torch.complex128 else 8
    K = GIB // (es * M)  # A occupies 1 GiB
    g = torch.Generator(device="cuda").manual_seed(64 + (1 if inplace else 0) + (2 if es == 16 else 0))
    A = uniform_dev(K * M, dtype, g)
    B = uniform_dev(M * N, dtype, g)
    C = A if inplace else uniform_dev(K * N, dtype, g)
    rows = torch.randint(0, K, (4096,), device="cuda", generator=g)
    A0 = A.view(K, M)[rows].cpu().numpy()
    C0 = C.view(K, N)[rows].cpu().numpy()
    Bh = B.cpu().numpy()
    handle.tsmm(M, N, K, A, M, 1.0, B, M, 0.5, C, N)
    got = C.view(K, N)[rows].cpu().numpy().ravel()
    exp, den = common.tsmm_expected(M, N, 4096, A0.ravel(), M, Bh, M, C0.ravel(), N, 1.0, 0.5)
    err = common.normwise(got, exp, den)
    np_dt = np.complex128 if es == 16 else np.float64
    assert err <= common.tol(np_dt, M), err
    del A, B, C
    free()


def _spread_dev(n, g):
    s = torch.rand(n, dtype=torch.float64, device="cuda", generator=g) + 1.0
    e = torch.randint(-20, 21, (n,), device="cuda", generator=g)
    sg = torch.randint(0, 2, (n,), device="cuda", generator=g) * 2 - 1
    return torch.ldexp(s * sg, e)


@pytest.mark.parametrize("gram", [False, True], ids=["AtB", "gram"])
def test_c3_tsmttsm_128_full_size_sampled_entries(handle, gram):
    from oracle import oracle as O
    M = N = 128
    K = 1 << 24
    g = torch.Generator(device="cuda").manual_seed(3128 + gram)
    A = _spread_dev(K * M, g)
    B = A if gram else _spread_dev(K * N, g)
    ms = torch.randperm(M, device="cuda", generator=g)[:8].sort().values
    ns = torch.randperm(N, device="cuda", generator=g)[:8].sort().values
    As = A.view(K, M)[:, ms].contiguous().cpu().numpy().ravel()
    Bs = B.view(K, N)[:, ns].contiguous().cpu().numpy().ravel()
    hi, lo = O.tsmttsm_exact(8, 8, K, As, 8, Bs, 8)
    den, _ = O.tsmttsm_exact(8, 8, K, np.abs(As), 8, np.abs(Bs), 8)
    exact = hi + lo  # exact[j*8+i] = C[ms[i], ns[j]]
    mi, nj = ms.cpu().numpy(), ns.cpu().numpy()
    idx = (nj[:, None] * M + mi[None, :]).ravel()  # C[n*ldc+m], ldc = M
    bounds = {"split": 1e-15, "native": common.tol(np.float64, K), "dd": 2.0 ** -52}
    for acc, bound in bounds.items():
        C = torch.zeros(M * N, dtype=torch.float64, device="cuda")
        handle.tsmttsm(M, N, K, A, M, 1.0, B, N, 0.0, C, M, acc=acc)
        got = C.cpu().numpy()[idx]
        err = float(np.linalg.norm(got - exact) / np.linalg.norm(den))
        assert err <= bound, (acc, err, bound)
    del A, B
    free()


def _make_x_dev(K, M, cond, seed):
    """X = G R on the device: G seeded standard Gaussian, R the triangular factor of
    U diag(sigma) V^T with sigma log-spaced from 1 to 1/cond (as oracle/svqb.make_x)."""
    rng = np.random.default_rng(seed)
    U, _ = np.linalg.qr(rng.standard_normal((M, M)))
    V, _ = np.linalg.qr(rng.standard_normal((M, M)))
    sig = np.logspace(0, -np.log10(cond), M)
    _, R = np.linalg.qr(U @ np.diag(sig) @ V.T)
    g = torch.Generator(device="cuda").manual_seed(seed)
    G = torch.randn(K, M, dtype=torch.float64, device="cuda", generator=g)
    return (G @ torch.from_numpy(R).cuda()).contiguous().view(-1)


@pytest.mark.parametrize("M", [16, 32, 64])
def test_c4_svqb_full_size_properties(handle, M):
    K = 1 << 24
    X0 = _make_x_dev(K, M, 1e8, seed=4000 + M)
    X = X0.clone()
    e1 = handle.svqb(K, M, X, M, gram_acc="split")
    e2 = handle.svqb(K, M, X, M, gram_acc="split")
    assert e2 <= 1e-12, (e1, e2)
    Q = X.view(K, M)
    S = torch.zeros(M * M, dtype=torch.float64, device="cuda")
    handle.tsmttsm(M, M, K, X, M, 1.0, X, M, 0.0, S, M, acc="dd")  # independent Gram, double-double
    orth = float(torch.linalg.norm(S.view(M, M) - torch.eye(M, dtype=torch.float64, device="cuda")))
    assert orth <= 1e-12 and abs(orth - e2) <= 1e-13 + 1e-3 * e2, (orth, e2)
    R = torch.zeros(M * M, dtype=torch.float64, device="cuda")
    handle.tsmttsm(M, M, K, X, M, 1.0, X0, M, 0.0, R, M, acc="split")  # R = Q^T X0 (C[n*M+m])
    Rm = R.view(M, M).T  # Rm[m, n] = (Q^T X0)[m, n]
    resid = float(torch.linalg.norm(X0.view(K, M) - Q @ Rm) / torch.linalg.norm(X0))
    assert resid <= 1e-9, resid
    del X0, X, Q
    free()


def test_c4_svqb_full_size_matches_host_oracle(handle):
    """K = 2^24, M = 64 at condition 1e3: one pass on the device against oracle/svqb.py with its
    FP64 loop Gram; the Grams differ by the FP64 loop's rounding (~sqrt(K) u relative), which the
    transform amplifies by the condition squared."""
    from oracle import svqb as OS
    K, M = 1 << 24, 64
    Xd = _make_x_dev(K, M, 1e3, seed=4100)
    X = Xd.cpu().numpy()
    handle.svqb(K, M, Xd, M, gram_acc="split", orth_err=False)
    Q = Xd.cpu().numpy()
    Qr = OS.svqb(X, K, M, "plain")
    Q2, R2 = Q.reshape(K, M), Qr.reshape(K, M)
    s = np.sign(np.sum(Q2[:65536] * R2[:65536], axis=0))
    rel = float(np.linalg.norm(Q2 * s[None, :] - R2) / np.linalg.norm(R2))
    bound = 1e3 ** 2 * 8 * math.sqrt(K) * 2.0 ** -53
    assert rel <= bound, (rel, bound)
    del Xd
    free()
