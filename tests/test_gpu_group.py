"""GPU tests of grouped launches (skinny_group): batches of small TSMTTSM / TSMM products of every
dtype in one launch, each item checked against the exact oracle within the working precision's
bound; TSMM items bit-identical to skinny_tsmm (same arithmetic order); TSMTTSM items
deterministic and independent of the rest of the batch; the integer fixtures bit-exact; argument
errors reported before anything runs."""
import numpy as np
import pytest

import common

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

from skinny_matmul_gb300 import lib as L  # noqa: E402

DTYPES = ["float32", "float64", "complex64", "complex128"]
NP = {"float32": np.float32, "float64": np.float64, "complex64": np.complex64, "complex128": np.complex128}


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def make_item(rng, dt, op, M, N, K, pad=0, beta=0.5, alpha=1.0, gram=False, inplace=False):
    """Host operands and device copies of one item (reference layouts, leading dimensions padded)."""
    npdt = NP[dt]
    u = lambda n: common.uniform(rng, n, npdt)
    if op == "tsmttsm":
        lda = M + pad
        ldb = lda if gram else N + pad
        ldc = M + pad
        A = u(K * lda)
        B = A if gram else u(K * ldb)
        C0 = u(N * ldc)
    else:
        lda = M + pad
        ldb = M + pad
        ldc = lda if inplace else N + pad
        A = u(K * lda)
        B = u(N * ldb)
        C0 = A if inplace else u(K * ldc)
    dA = dev(A)
    dB = dA if (op == "tsmttsm" and gram) else dev(B)
    dC = dA if inplace else dev(C0)
    return dict(op=op, M=M, N=N, K=K, A=dA, lda=lda, B=dB, ldb=ldb, C=dC, ldc=ldc, alpha=alpha, beta=beta,
                hA=A, hB=B, hC0=C0.copy(), dt=dt)


def check(it):
    got = host(it["C"])
    M, N, K, dt = it["M"], it["N"], it["K"], it["dt"]
    if it["op"] == "tsmttsm":
        exp, den = common.tsmttsm_expected(M, N, K, it["hA"], it["lda"], it["hB"], it["ldb"], it["hC0"], it["ldc"],
                                           it["alpha"], it["beta"])
        mask = common.c_mask_tsmttsm(M, N, it["ldc"])
        bound = common.tol(NP[dt], K)
    else:
        exp, den = common.tsmm_expected(M, N, K, it["hA"], it["lda"], it["hB"], it["ldb"], it["hC0"], it["ldc"],
                                        it["alpha"], it["beta"])
        mask = common.c_mask_tsmm(N, K, it["ldc"])
        bound = common.tol(NP[dt], M)
    err = common.normwise(got, exp, den, mask)
    assert err <= bound, (it["op"], dt, M, N, K, it["lda"], err, bound)


def random_batch(rng, dt, n, kmax=6000):
    items = []
    for i in range(n):
        op = "tsmttsm" if rng.random() < 0.55 else "tsmm"
        M = int(rng.choice([1, 2, 3, 4, 5, 8, 13, 16, 31, 32, 47, 64]))
        N = int(rng.choice([1, 2, 3, 4, 5, 8, 13, 16, 31, 32, 47, 64]))
        K = int(rng.choice([0, 1, 17, 129, 1000, kmax])) if op == "tsmttsm" else int(rng.choice([1, 17, 1000, kmax]))
        K = min(K, max(1, 2_000_000 // (M * N)))  # keeps the exact oracle quick
        pad = int(rng.choice([0, 0, 1, 3]))
        beta = float(rng.choice([0.0, 0.5]))
        alpha = 1.0 if rng.random() < 0.5 else (-0.75 + (0.25j if dt.startswith("complex") else 0))
        gram = op == "tsmttsm" and M == N and rng.random() < 0.4
        inplace = op == "tsmm" and M == N and rng.random() < 0.4
        items.append(make_item(rng, dt, op, M, N, K, pad, beta, alpha, gram, inplace))
    return items


@pytest.mark.parametrize("dt", DTYPES)
def test_group_batch_matches_oracle(handle, dt):
    rng = np.random.default_rng(100 + DTYPES.index(dt))
    items = random_batch(rng, dt, 28)
    handle.group(items, dtype=dt)
    for it in items:
        check(it)


@pytest.mark.parametrize("dt", DTYPES)
def test_group_tsmm_bitwise_equals_single_launch(handle, dt):
    rng = np.random.default_rng(7)
    items = [make_item(rng, dt, "tsmm", M, N, K, pad, beta, alpha, inplace=ip)
             for (M, N, K, pad, beta, alpha, ip) in [(1, 1, 70001, 0, 0.5, 1.0, False), (4, 16, 5000, 1, 0.0, 2.0, False),
                                                     (16, 4, 3000, 0, 0.5, 1.0, True), (8, 32, 2000, 0, 0.5, -1.0, False),
                                                     (64, 64, 700, 2, 0.5, 1.0, True), (3, 5, 999, 0, 0.5, 1.0, False)]]
    singles = []
    for it in items:
        C = dev(it["hC0"]) if it["C"] is not it["A"] else dev(it["hA"])
        A = C if it["C"] is it["A"] else it["A"]
        handle.tsmm(it["M"], it["N"], it["K"], A, it["lda"], it["alpha"], it["B"], it["ldb"], it["beta"], C,
                    it["ldc"], acc="native", dtype={"float32": L.R32, "float64": L.R64, "complex64": L.C32,
                                                    "complex128": L.C64}[dt])
        singles.append(C)
    handle.group(items, dtype=dt)
    for it, s in zip(items, singles):
        assert np.array_equal(host(it["C"]), host(s)), (dt, it["M"], it["N"], it["K"])
        check(it)


def test_group_tsmttsm_independent_of_batch_and_deterministic(handle):
    rng = np.random.default_rng(3)
    probe = make_item(rng, "float64", "tsmttsm", 16, 16, 40000, beta=0.0)
    handle.group([probe], dtype="float64")
    alone = host(probe["C"]).copy()
    others = random_batch(np.random.default_rng(4), "float64", 40)
    for pos in (0, 17, 40):
        batch = others[:pos] + [probe] + others[pos:]
        handle.group(batch, dtype="float64")
        assert np.array_equal(host(probe["C"]), alone), pos
    check(probe)


@pytest.mark.parametrize("case", list(common.int_cases()), ids=lambda c: c["id"])
def test_group_integer_fixtures_bit_exact(handle, case):
    c = case
    if c["M"] > 64 or c["N"] > 64:
        pytest.skip("grouped items are at most 64 wide")
    for dt in (["complex64", "complex128"] if c["cplx"] else ["float32", "float64"]):
        A = dev(c["A"].astype(NP[dt]))
        B = dev(c["B"].astype(NP[dt]))
        C = dev(c["C"].astype(NP[dt]))
        if c["self"] and c["op"] == "tsmttsm":
            B = A
        if c["self"] and c["op"] == "tsmm":
            A = C
        handle.group([dict(op=c["op"], M=c["M"], N=c["N"], K=c["K"], A=A, lda=c["lda"], B=B, ldb=c["ldb"], C=C,
                           ldc=c["ldc"], alpha=1.0, beta=float(c["beta"]))], dtype=dt)
        got = host(C).astype(np.complex128 if c["cplx"] else np.float64)
        assert np.array_equal(got, c["exp"]), dt


def test_group_many_items_one_launch(handle):
    rng = np.random.default_rng(9)
    items = []
    for i in range(1500):
        op = "tsmttsm" if i % 2 == 0 else "tsmm"
        M, N = int(rng.integers(1, 9)), int(rng.integers(1, 9))
        items.append(make_item(rng, "float64", op, M, N, int(rng.integers(1, 3000)), beta=0.5))
    n0 = L.load().skinny_kernel_launches()
    handle.group(items, dtype="float64")
    assert L.load().skinny_kernel_launches() - n0 == 1
    for it in items[::7]:
        check(it)


def test_group_on_a_side_stream(handle):
    rng = np.random.default_rng(12)
    items = random_batch(rng, "complex128", 10)
    s = torch.cuda.Stream()
    torch.cuda.synchronize()
    with torch.cuda.stream(s):
        handle.group(items, dtype="complex128", stream=s)
    s.synchronize()
    for it in items:
        check(it)


def test_group_argument_errors(handle):
    rng = np.random.default_rng(1)
    ok = make_item(rng, "float64", "tsmttsm", 4, 4, 100)
    wide = make_item(rng, "float64", "tsmttsm", 65, 4, 10)
    with pytest.raises(L.SkinnyError) as e:
        handle.group([ok, wide], dtype="float64")
    assert e.value.status == L.UNSUPPORTED
    bad_ld = dict(ok, lda=3)
    with pytest.raises(L.SkinnyError) as e:
        handle.group([bad_ld], dtype="float64")
    assert e.value.status == L.BAD_ARG
    misaligned = dict(ok, A=ok["A"].data_ptr() + 4, B=ok["B"].data_ptr())
    with pytest.raises(L.SkinnyError) as e:
        handle.group([misaligned], dtype="float64")
    assert e.value.status == L.BAD_ARG
    svqb = dict(ok, op="svqb")
    with pytest.raises(L.SkinnyError) as e:
        handle.group([svqb], dtype="float64")
    assert e.value.status == L.BAD_ARG
