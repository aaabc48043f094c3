"""Failure detection without a GPU fault: a bounded device-side wait that runs out.

The CUDA-core TSMTTSM ring kernel (products wider than 8, or above the row-streaming kernel's
register tile) waits on mbarriers for the bulk copies of its row ring.  With the
handle's poll limit set to 0 every such wait gives up at once; the kernel records SKINNY_TIMEOUT
in the handle's device error word, waits (with the default bound) for the copies it has already
issued, and exits without writing C.  The host reads the status with skinny_check_device, which
also resets the ticket counters, and the next call with the default limit is correct.
Nothing here traps, faults or hangs the GPU: every wait is bounded and every issued copy lands.
"""
import numpy as np
import pytest

import common

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def test_wait_timeout_is_reported_and_the_next_call_is_correct():
    from skinny_matmul_gb300 import Handle, SkinnyError, build
    build.build()
    h = Handle(0)
    try:
        rng = np.random.default_rng(11)
        M = N = 16  # the ring kernel (narrower products stream rows without waits)
        K = 1 << 18  # many full row tiles per CTA: the ring is fed by bulk copies
        A = rng.uniform(-1, 1, K * M)
        B = rng.uniform(-1, 1, K * N)
        Ad, Bd = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
        C = torch.full((M * N,), 7.0, dtype=torch.float64, device="cuda")
        h.set_wait_limit(0)
        h.tsmttsm(M, N, K, Ad, M, 1.0, Bd, N, 0.0, C, M, acc="native")
        with pytest.raises(SkinnyError, match="TIMEOUT"):
            h.check_device()
        assert torch.all(C == 7.0).item(), "a timed-out launch must not write C"
        h.check_device()  # the flag was cleared by the previous check

        h.set_wait_limit(1 << 22)
        for _ in range(2):
            h.tsmttsm(M, N, K, Ad, M, 1.0, Bd, N, 0.0, C, M, acc="native")
            torch.cuda.synchronize()
            exp, den = common.tsmttsm_expected(M, N, K, A, M, B, N, np.zeros(M * N), M, 1.0, 0.0)
            assert common.normwise(C.cpu().numpy(), exp, den) <= common.tol(np.float64, K)
        h.check_device()
    finally:
        h.close()


def test_gram_and_float_paths_recover_after_timeouts():
    from skinny_matmul_gb300 import Handle, SkinnyError, build
    build.build()
    h = Handle(0)
    try:
        rng = np.random.default_rng(12)
        for dt, M in ((np.float64, 16), (np.float32, 16)):
            K = 300007
            X = rng.uniform(-1, 1, K * M).astype(dt)
            Xd = torch.from_numpy(X).cuda()
            S = torch.zeros(M * M, dtype=Xd.dtype, device="cuda")
            h.set_wait_limit(0)
            h.tsmttsm(M, M, K, Xd, M, 1.0, Xd, M, 0.0, S, M, acc="native")  # Gram mode
            with pytest.raises(SkinnyError, match="TIMEOUT"):
                h.check_device()
            h.set_wait_limit(1 << 22)
            h.tsmttsm(M, M, K, Xd, M, 1.0, Xd, M, 0.0, S, M, acc="native")
            torch.cuda.synchronize()
            exp, den = common.tsmttsm_expected(M, M, K, X.astype(np.float64), M, X.astype(np.float64), M,
                                               np.zeros(M * M), M, 1.0, 0.0)
            assert common.normwise(S.cpu().numpy(), exp, den) <= common.tol(dt, K), dt
        h.check_device()
    finally:
        h.close()
