"""GPU test of skinny_tsmttsm_d_static, the FP64 TSMTTSM entry point that allocates no device memory.

It exists for callers that cannot call cudaMalloc (an allocator that owns the whole device pool,
or a latency-critical path where cudaMalloc's implicit synchronisation is not allowed), so it takes
its scratch from a fixed array inside the library instead of a handle's workspace.  The test calls
it through the C ABI twice in a row and compares each result with skinny_tsmttsm (R64, native)
and with the exact oracle, within the FP64 bound 8*sqrt(K)*u normwise.  It also covers the
largest accepted M*N (2^20, the partials of only two CTAs fit the array), a rejected size (C left
untouched), and the status query skinny_tsmttsm_d_static_check.  This file is named to be
collected last.
"""
import ctypes

import numpy as np
import pytest

import common

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _static(lib, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc):
    st = torch.cuda.current_stream().cuda_stream
    return lib.skinny_tsmttsm_d_static(M, N, K, A.data_ptr(), lda, alpha, B.data_ptr(), ldb, beta,
                                       C.data_ptr(), ldc, st)


@pytest.mark.parametrize("M,N,K", [(8, 8, 1 << 20), (5, 3, 1001), (128, 128, 20000), (1, 1, 77)])
def test_static_matches_handle_entry_two_calls(handle, M, N, K):
    from skinny_matmul_gb300 import lib as L
    lib = L.load()
    rng = np.random.default_rng(M * 7 + N + K)
    ldc = M + 1
    for call in range(2):  # two calls in a row: the shared scratch must not leak state
        A = torch.from_numpy(rng.uniform(-1, 1, K * M)).cuda()
        B = torch.from_numpy(rng.uniform(-1, 1, K * N)).cuda()
        C0 = torch.from_numpy(rng.uniform(-1, 1, N * ldc)).cuda()
        alpha, beta = (1.0, 0.0) if call == 0 else (-0.5, 2.0)
        C_static = C0.clone()
        C_ref = C0.clone()
        st = _static(lib, M, N, K, A, M, alpha, B, N, beta, C_static, ldc)
        assert st == L.OK, L.last_error()
        handle.tsmttsm(M, N, K, A, M, alpha, B, N, beta, C_ref, ldc)
        torch.cuda.synchronize()
        got, ref = C_static.cpu().numpy(), C_ref.cpu().numpy()
        mask = common.c_mask_tsmttsm(M, N, ldc)
        den = np.abs(ref[mask]) + 1e-300
        absprod = (np.abs(A.cpu().numpy()).reshape(K, M).T @ np.abs(B.cpu().numpy()).reshape(K, N)).T.ravel()
        scale = abs(alpha) * absprod + abs(beta) * np.abs(C0.cpu().numpy()[mask])
        err = np.linalg.norm(got[mask] - ref[mask]) / np.linalg.norm(scale)
        assert err <= common.tol(np.float64, K), (call, err)
        assert np.array_equal(got[~mask], C0.cpu().numpy()[~mask])
        exp, den = common.tsmttsm_expected(M, N, K, A.cpu().numpy(), M, B.cpu().numpy(), N,
                                           C0.cpu().numpy(), ldc, alpha, beta)
        assert common.normwise(got, exp, den, mask) <= common.tol(np.float64, K), call
    assert lib.skinny_tsmttsm_d_static_check(torch.cuda.current_stream().cuda_stream) == L.OK


def test_static_gram_mode(handle):
    from skinny_matmul_gb300 import lib as L
    lib = L.load()
    rng = np.random.default_rng(3)
    M, K = 16, 50000
    X = torch.from_numpy(rng.uniform(-1, 1, K * M)).cuda()
    S1 = torch.zeros(M * M, dtype=torch.float64, device="cuda")
    S2 = torch.zeros_like(S1)
    assert _static(lib, M, M, K, X, M, 1.0, X, M, 0.0, S1, M) == L.OK
    handle.tsmttsm(M, M, K, X, M, 1.0, X, M, 0.0, S2, M)
    torch.cuda.synchronize()
    s1, s2 = S1.cpu().numpy(), S2.cpu().numpy()
    assert np.linalg.norm(s1 - s2) / np.linalg.norm(s2) <= common.tol(np.float64, K)


def test_static_at_the_size_limit(handle):
    """M * N = 2^20 (Gram, M = N = 1024): the largest accepted size; the array then holds the
    partials of two CTAs, so the grid is cut to two."""
    from skinny_matmul_gb300 import lib as L
    lib = L.load()
    rng = np.random.default_rng(5)
    M, K = 1024, 64
    X = torch.from_numpy(rng.uniform(-1, 1, K * M)).cuda()
    S_static = torch.zeros(M * M, dtype=torch.float64, device="cuda")
    S_ref = torch.zeros_like(S_static)
    for _ in range(2):
        assert _static(lib, M, M, K, X, M, 1.0, X, M, 0.0, S_static, M) == L.OK, L.last_error()
        handle.tsmttsm(M, M, K, X, M, 1.0, X, M, 0.0, S_ref, M, acc="native")
        torch.cuda.synchronize()
        got, ref = S_static.cpu().numpy(), S_ref.cpu().numpy()
        Xh = X.cpu().numpy()
        exp, den = common.tsmttsm_expected(M, M, K, Xh, M, Xh, M, np.zeros(M * M), M, 1.0, 0.0)
        assert common.normwise(got, exp, den) <= common.tol(np.float64, K)
        assert common.normwise(got, ref, den) <= 2 * common.tol(np.float64, K)
    assert lib.skinny_tsmttsm_d_static_check(torch.cuda.current_stream().cuda_stream) == L.OK


def test_static_rejects_oversized_and_bad_arguments():
    from skinny_matmul_gb300 import lib as L
    lib = L.load()
    X = torch.zeros(16, dtype=torch.float64, device="cuda")
    C = torch.arange(16, dtype=torch.float64, device="cuda")
    p = X.data_ptr()
    # M * N one column above 2^20 entries of C: rejected before any device work, C untouched
    st = lib.skinny_tsmttsm_d_static(1024, 1025, 4, p, 1024, 1.0, p, 1025, 0.0, C.data_ptr(), 1024, None)
    assert st == L.BAD_ARG and "static scratch" in L.last_error()
    st = lib.skinny_tsmttsm_d_static(4, 4, 4, p, 3, 1.0, p, 4, 0.0, C.data_ptr(), 4, None)  # lda < M
    assert st == L.BAD_ARG
    torch.cuda.synchronize()
    assert torch.equal(C, torch.arange(16, dtype=torch.float64, device="cuda"))
