"""GPU tests of the request loop: a mixed stream of TSMTTSM / TSMM / SVQB requests in FP64,
complex FP64 and FP32 runs through the server with several requests in flight, and every result
is bit-identical to the same request run alone (the kernels are deterministic), and within the
working precision's bound of the oracle.  With grouping on, small requests run in grouped
launches replayed from CUDA graphs; each of their results is bit-identical to the same item in a
grouped launch of its own."""
import numpy as np
import pytest

import common

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

from skinny_matmul_gb300 import lib as L  # noqa: E402
from skinny_matmul_gb300.api import Server  # noqa: E402


def make_requests(seed, n):
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(n):
        op = rng.choice(["tsmttsm", "tsmm", "svqb"], p=[0.5, 0.35, 0.15])
        dtype = rng.choice(["float64", "complex128", "float32"], p=[0.6, 0.25, 0.15])
        if op == "svqb":
            dtype = "float64"
        K = int(2 ** rng.uniform(10, 16))
        M = int(rng.choice([1, 2, 4, 8, 16]))
        N = int(rng.choice([1, 2, 4, 8, 16])) if op != "svqb" else M
        npdt = {"float64": np.float64, "complex128": np.complex128, "float32": np.float32}[dtype]
        u = lambda n_: common.uniform(rng, n_, npdt)
        if op == "tsmttsm":
            gram = M == N and rng.random() < 0.3
            A = u(K * M)
            B = A if gram else u(K * N)
            C = u(N * M)
            r = dict(op=op, dtype=dtype, M=M, N=N, K=K, A=A, lda=M, B=B, ldb=M if gram else N, C=C, ldc=M,
                     alpha=1.0, beta=float(rng.choice([0.0, 0.5])))
        elif op == "tsmm":
            inplace = M == N and rng.random() < 0.3
            A = u(K * M)
            B = u(M * N)
            C = A if inplace else u(K * N)
            r = dict(op=op, dtype=dtype, M=M, N=N, K=K, A=A, lda=M, B=B, ldb=M, C=C, ldc=M if inplace else N,
                     alpha=1.0, beta=0.5)
        else:
            from oracle import svqb as OS
            X = OS.make_x(K, M, 1e2, seed=i)
            r = dict(op=op, dtype=dtype, M=M, N=M, K=K, A=X, lda=M, B=None, ldb=0, C=X, ldc=M, alpha=1.0, beta=0.0)
        r["acc"] = "native"
        reqs.append(r)
    return reqs


def run_alone(handle, r):
    """The same request through the handle API, device buffers via torch."""
    A = torch.from_numpy(r["A"].copy()).cuda()
    if r["op"] == "svqb":
        handle.svqb(r["K"], r["M"], A, r["lda"], gram_acc=r["acc"], orth_err=False)
        torch.cuda.synchronize()
        return A.cpu().numpy()
    same_ab = r["B"] is r["A"]
    same_ac = r["C"] is r["A"]
    B = A if same_ab else torch.from_numpy(r["B"].copy()).cuda()
    C = A if same_ac else torch.from_numpy(r["C"].copy()).cuda()
    fn = handle.tsmttsm if r["op"] == "tsmttsm" else handle.tsmm
    fn(r["M"], r["N"], r["K"], A, r["lda"], r["alpha"], B, r["ldb"], r["beta"], C, r["ldc"], acc=r["acc"])
    torch.cuda.synchronize()
    return C.cpu().numpy()


def test_mixed_stream_identical_alone_and_in_the_mix(handle):
    reqs = make_requests(11, 60)
    expected = [run_alone(handle, r) for r in reqs]
    srv = Server(handle, 2 << 30, num_streams=4, max_inflight=12, group_bytes=0)
    tickets = []
    for r in reqs:
        if r["op"] == "svqb":
            r["A"] = r["A"].copy()
            r["C"] = r["A"]
        elif r["C"] is r["A"]:
            r["A"] = r["A"].copy()
            r["C"] = r["A"]
            r["B"] = r["B"].copy()
        else:
            r["C"] = r["C"].copy()
        st, t = srv.submit(r["op"], r["dtype"], r["M"], r["N"], r["K"], r["A"], r["lda"], r["B"], r["ldb"],
                           r["C"], r["ldc"], r["alpha"], r["beta"], r["acc"])
        assert st == L.OK
        tickets.append(t)
    for t in tickets:
        st, res = srv.wait(t, 120)
        assert st == L.OK and res == L.OK
    stats = srv.stats()
    assert stats["completed"] == len(reqs) and stats["max_inflight_seen"] >= 2
    for r, e in zip(reqs, expected):
        assert np.array_equal(r["C"], e), (r["op"], r["dtype"], r["M"], r["N"], r["K"])
    srv.close()


def test_served_results_match_oracle(handle):
    reqs = [r for r in make_requests(5, 30) if r["op"] == "tsmttsm" and r["dtype"] == "float64"][:6]
    srv = Server(handle, 1 << 30)  # grouping on (default): these small requests run grouped
    outs = []
    for r in reqs:
        C = r["C"].copy()
        C0 = r["C"].copy()
        st, t = srv.submit("tsmttsm", "float64", r["M"], r["N"], r["K"], r["A"], r["lda"], r["B"], r["ldb"], C,
                           r["ldc"], r["alpha"], r["beta"])
        outs.append((t, C, C0, r))
    for t, C, C0, r in outs:
        assert srv.wait(t, 60) == (L.OK, L.OK)
        exp, den = common.tsmttsm_expected(r["M"], r["N"], r["K"], r["A"], r["lda"], r["B"], r["ldb"], C0, r["ldc"],
                                           r["alpha"], r["beta"])
        assert common.normwise(C, exp, den, common.c_mask_tsmttsm(r["M"], r["N"], r["ldc"])) <= \
            common.tol(np.float64, r["K"])
    srv.close()


def test_device_resident_requests_identical_to_alone(handle):
    """Requests on operands resident in HBM (device flag): the server runs them in place, several
    in flight; every result equals the same request run alone."""
    reqs = make_requests(23, 40)
    expected = [run_alone(handle, r) for r in reqs]
    srv = Server(handle, 8 << 30, num_streams=4, max_inflight=8, group_bytes=0)
    outs, tickets = [], []
    for r in reqs:
        A = torch.from_numpy(r["A"].copy()).cuda()
        if r["op"] == "svqb":
            B, C = None, A
        else:
            B = A if r["B"] is r["A"] else torch.from_numpy(r["B"].copy()).cuda()
            C = A if r["C"] is r["A"] else torch.from_numpy(r["C"].copy()).cuda()
        outs.append((A, B, C))
        st, t = srv.submit(r["op"], r["dtype"], r["M"], r["N"], r["K"], A, r["lda"], B, r["ldb"], C, r["ldc"],
                           r["alpha"], r["beta"], r["acc"], device=True)
        assert st == L.OK
        tickets.append(t)
    for t in tickets:
        assert srv.wait(t, 120) == (L.OK, L.OK)
    stats = srv.stats()
    assert stats["completed"] == len(reqs) and stats["max_inflight_seen"] >= 2
    for (A, B, C), r, e in zip(outs, reqs, expected):
        assert np.array_equal(C.cpu().numpy(), e), (r["op"], r["dtype"], r["M"], r["N"], r["K"])
    srv.close()


def _group_alone(handle, r):
    """The same request as the only item of a grouped launch (device buffers via torch)."""
    A = torch.from_numpy(r["A"].copy()).cuda()
    B = A if r["B"] is r["A"] else torch.from_numpy(r["B"].copy()).cuda()
    C = A if r["C"] is r["A"] else torch.from_numpy(r["C"].copy()).cuda()
    handle.group([dict(op=r["op"], M=r["M"], N=r["N"], K=r["K"], A=A, lda=r["lda"], B=B, ldb=r["ldb"], C=C,
                       ldc=r["ldc"], alpha=r["alpha"], beta=r["beta"])], dtype=r["dtype"])
    torch.cuda.synchronize()
    return C.cpu().numpy()


@pytest.mark.parametrize("device", [False, True])
def test_grouped_requests_identical_to_their_own_group(handle, device):
    """Small requests (host or device operands) packed into graph-replayed grouped launches give
    the bits of the same item alone in a grouped launch; large and SVQB requests still run on
    their own in the same stream."""
    reqs = make_requests(31 + device, 80)
    expected = []
    for r in reqs:
        if r["op"] == "svqb":
            expected.append(run_alone(handle, r))
        else:
            expected.append(_group_alone(handle, r))
    # a threshold above every request's cost: every TSMTTSM / TSMM request runs grouped
    srv = Server(handle, 4 << 30, num_streams=4, max_inflight=8, group_bytes=1 << 40, group_max=64)
    outs, tickets = [], []
    for r in reqs:
        if device:
            A = torch.from_numpy(r["A"].copy()).cuda()
            if r["op"] == "svqb":
                B, C = None, A
            else:
                B = A if r["B"] is r["A"] else torch.from_numpy(r["B"].copy()).cuda()
                C = A if r["C"] is r["A"] else torch.from_numpy(r["C"].copy()).cuda()
        else:
            A = r["A"].copy()
            B = None if r["op"] == "svqb" else (A if r["B"] is r["A"] else r["B"].copy())
            C = A if (r["op"] == "svqb" or r["C"] is r["A"]) else r["C"].copy()
        outs.append((A, B, C))
        st, t = srv.submit(r["op"], r["dtype"], r["M"], r["N"], r["K"], A, r["lda"], B, r["ldb"], C, r["ldc"],
                           r["alpha"], r["beta"], r["acc"], device=device)
        assert st == L.OK
        tickets.append(t)
    for t in tickets:
        assert srv.wait(t, 120) == (L.OK, L.OK)
    stats = srv.stats()
    n_small = sum(r["op"] != "svqb" for r in reqs)
    assert stats["completed"] == len(reqs)
    assert stats["grouped"] == n_small
    assert 1 <= stats["group_launches"] <= n_small
    for (A, B, C), r, e in zip(outs, reqs, expected):
        got = C.cpu().numpy() if device else C
        assert np.array_equal(got, e), (r["op"], r["dtype"], r["M"], r["N"], r["K"])
    srv.close()
