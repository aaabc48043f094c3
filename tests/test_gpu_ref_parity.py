"""Parity with the REFERENCE's own kernels, run on the same GPU on the same seeded inputs.

The reference's kernels (GENV5, GENV3X, SPECSMALL with double and PseudoQuad accumulation, FIX3,
FIX_FB, FIX_IP_GHOST) are compiled from its headers for sm_103a by `make -C oracle ref` and
launched with its launchers' configuration by oracle/ref_runner.cpp.  This library is called
through its C ABI on the same device buffers.

Bars (written into each assertion):
  * golden integer cases (the test.cu fixture design, test.cu:65-103, 247-276): every reference
    kernel and every method of this library bit-exact, and equal to the fixture's exact value;
  * seeded U[-1,1) data (C1: TSMTTSM FP64 8x8, K = 2^20; the small C2 widths of TSMM, alpha 1,
    beta 0.5): each side within 8 sqrt(K) u normwise of the exact oracle (K for TSMTTSM, M for
    TSMM), and the two sides within twice that of each other;
  * double-double: this library's `dd` method against SPECSMALL<double, PseudoQuad> (plus the
    reduction of specsmall.cuh:10-26) on the numeric_tests.cu:58-61 cancellation test.

Comparisons with kernels the reference runs with intra-warp shared-memory races (SPECSMALL's row
cache, specsmall.cuh:56-66; GENV5's row cache, genv5.cuh:59-64) are informational where they
disagree: such a disagreement is reported, not asserted, unless this library also disagrees with
the exact value.  GENV6 is not run: its kernel reads past its shared B cache (genv6.cuh:54)
once K reaches its rows per block, which faulted on GB300.
"""
import math

import numpy as np
import pytest

import common

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

TS_VARIANTS = [("GENV5", "float64"), ("GENV3X", "float64"), ("SPECSMALL", "float64"),
               ("SPECSMALL_PQ", "float64"), ("GENV5", "float32"), ("SPECSMALL", "float32")]
RACY = {"SPECSMALL", "SPECSMALL_PQ", "GENV5"}
NP = {"float32": np.float32, "float64": np.float64, "complex128": np.complex128}
TD = {"float32": torch.float32, "float64": torch.float64, "complex128": torch.complex128}


@pytest.fixture(scope="module")
def ref():
    from oracle import ref_gpu
    if not ref_gpu.built():
        pytest.skip("reference kernels not built here (no reference tree when oracle/_ref was made)")
    msg = ref_gpu.init()
    assert msg is None, msg
    return ref_gpu


def put(ref, arr, dtype):
    """Device copy of a flat array, with the padding the reference kernels' over-reads need."""
    t = ref.padded(arr.size, TD[dtype])
    t.copy_(torch.from_numpy(np.ascontiguousarray(arr.astype(NP[dtype]))))
    return t


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def test_reference_kernels_loaded(ref):
    names = ref.kernel_names()
    for k in ("GENV5::blockProductKernel<double, 8, 8, 256, false>", "GENV5::deviceReduce<double, 8, 8>",
              "SPECSMALL::deviceReduce<double, PseudoQuad, 1, 1>", "tsmm_fix3_kernel<double, 64, 64, 256, false>",
              "fix_ip_ghost_kernel<double2, 8, 8>"):
        assert k in names, (k, names[:20])
    assert len(names) >= 200


TS_CASES = [c for c in common.int_cases() if c["op"] == "tsmttsm" and not c["cplx"]]
TSMM_CASES = [c for c in common.int_cases() if c["op"] == "tsmm"]


def _race_or_fail(variant, what):
    """A reference kernel with an intra-warp race disagreeing is reported, not failed."""
    if variant in RACY:
        pytest.xfail(f"reference kernel {variant} (intra-warp shared-memory race) disagrees: {what}")
    raise AssertionError(f"{variant}: {what}")


@pytest.mark.parametrize("case", TS_CASES, ids=lambda c: c["id"])
def test_tsmttsm_integer_fixtures_match_reference_kernels(ref, handle, case):
    c = case
    rng = np.random.default_rng(int(c["id"][1:]))
    ran, racy = [], []
    for variant, dt in TS_VARIANTS:
        bc = int(rng.integers(1, 201))  # test.cu:254 draws blockCount from [1, 200]
        A = put(ref, c["A"], dt)
        B = A if c["self"] else put(ref, c["B"], dt)
        ldb = c["lda"] if c["self"] else c["ldb"]
        C = put(ref, c["C"], dt)
        if not ref.tsmttsm(variant, c["M"], c["N"], c["K"], A, c["lda"], 1.0, B, ldb, float(c["beta"]), C,
                           c["ldc"], bc, dtype=dt):
            continue
        got = host(C).astype(np.float64)
        if not np.array_equal(got, c["exp"]):
            racy.append((variant, dt, bc))
        ran.append(variant)
        # this library on the same buffers and arguments: the fixture's exact value, bit for bit
        for acc in (("native", "auto", "dd") if dt == "float64" else ("native",)):
            C2 = put(ref, c["C"], dt)
            handle.tsmttsm(c["M"], c["N"], c["K"], A, c["lda"], 1.0, B, ldb, float(c["beta"]), C2, c["ldc"],
                           acc=acc)
            assert np.array_equal(host(C2).astype(np.float64), c["exp"]), (variant, dt, acc)
    if max(c["M"], c["N"]) <= 32:
        assert "GENV5" in ran and "SPECSMALL" in ran, ran
    for variant, dt, bc in racy:
        _race_or_fail(variant, f"{dt}, blockCount {bc}, integer fixture not reproduced")


@pytest.mark.parametrize("case", TSMM_CASES, ids=lambda c: c["id"])
def test_tsmm_integer_fixtures_match_reference_kernels(ref, handle, case):
    c = case
    rng = np.random.default_rng(1000 + int(c["id"][1:]))
    if c["cplx"]:
        variants = [("FIX_IP_GHOST", "complex128")] if c["self"] else []
    elif c["self"]:
        variants = [("FIX3", "float64"), ("FIX_IP_GHOST", "float64"), ("FIX3", "float32")]
    else:
        variants = [("FIX3", "float64"), ("FIX_FB", "float64"), ("FIX3", "float32")]
    if not variants:
        pytest.skip("the reference has no complex out-of-place TSMM kernel among those built (FIX1/VAR1)")
    ran = []
    for variant, dt in variants:
        bc = int(rng.integers(1, 201))
        C = put(ref, c["C"], dt)
        A = C if c["self"] else put(ref, c["A"], dt)
        lda = c["ldc"] if c["self"] else c["lda"]
        B = put(ref, c["B"], dt)
        if not ref.tsmm(variant, c["M"], c["N"], c["K"], A, lda, 1.0, B, c["ldb"], float(c["beta"]), C, c["ldc"],
                        bc, dtype=dt):
            continue
        got = host(C).astype(np.complex128 if c["cplx"] else np.float64)
        assert np.array_equal(got, c["exp"]), (variant, dt, bc)
        ran.append(variant)
        C2 = put(ref, c["C"], dt)
        A2 = C2 if c["self"] else A
        handle.tsmm(c["M"], c["N"], c["K"], A2, lda, 1.0, B, c["ldb"], float(c["beta"]), C2, c["ldc"])
        assert np.array_equal(host(C2), host(C)), (variant, dt)
    assert ran, variants


def _normwise(got, exp, den, mask):
    return common.normwise(got, exp, den, mask)


@pytest.fixture(scope="module")
def c1_data():
    """C1: TSMTTSM FP64 8 x 8, K = 2^20, U[-1,1), alpha 1, beta 0, with the exact oracle's C."""
    rng = np.random.default_rng(20260101)
    M = N = 8
    K = 1 << 20
    A = rng.uniform(-1, 1, K * M)
    B = rng.uniform(-1, 1, K * N)
    exp, den = common.tsmttsm_expected(M, N, K, A, M, B, N, np.zeros(M * N), M, 1.0, 0.0)
    return M, N, K, A, B, exp, den


@pytest.mark.parametrize("variant", ["GENV5", "GENV3X", "SPECSMALL", "SPECSMALL_PQ"])
def test_c1_random_against_reference_kernel(ref, handle, c1_data, variant):
    M, N, K, A, B, exp, den = c1_data
    Ad, Bd = put(ref, A, "float64"), put(ref, B, "float64")
    Cr = put(ref, np.zeros(M * N), "float64")
    assert ref.tsmttsm(variant, M, N, K, Ad, M, 1.0, Bd, N, 0.0, Cr, M, 1024)
    ref_c = host(Cr)
    bound = common.tol(np.float64, K)  # 8 sqrt(K) 2^-53
    mask = np.ones(M * N, dtype=bool)
    e_ref = _normwise(ref_c, exp, den, mask)
    ours_ok = []
    for acc in ("native", "split", "auto", "dd"):
        Co = put(ref, np.zeros(M * N), "float64")
        handle.tsmttsm(M, N, K, Ad, M, 1.0, Bd, N, 0.0, Co, M, acc=acc)
        ours = host(Co)
        e_ours = _normwise(ours, exp, den, mask)
        assert e_ours <= bound, (acc, e_ours, bound)
        ours_ok.append((acc, ours))
    if e_ref > bound:
        _race_or_fail(variant, f"normwise error {e_ref:.3g} > {bound:.3g}")
    for acc, ours in ours_ok:
        diff = _normwise(ours, ref_c, den, mask)
        assert diff <= 2 * bound, (variant, acc, diff)
        if variant == "SPECSMALL_PQ" and acc == "dd":
            # both accumulate in double-double and round once to FP64: within the output rounding
            assert diff <= 2.0 ** -51, diff


TSMM_SHAPES = [(1, 1), (2, 2), (4, 4), (8, 8), (16, 16), (32, 32), (64, 64), (4, 16), (16, 4), (8, 32)]


@pytest.mark.parametrize("M,N", TSMM_SHAPES)
@pytest.mark.parametrize("inplace", [False, True])
def test_c2_widths_random_against_reference_kernels(ref, handle, M, N, inplace):
    """C2 widths, FP64, alpha 1, beta 0.5 (K = 20011 rows; the bound does not depend on K)."""
    if inplace and M != N:
        pytest.skip("C2's in-place form has M = N")
    rng = np.random.default_rng(M * 100 + N + (7 if inplace else 0))
    K = 20011
    ld = max(M, N) if inplace else None
    lda, ldb, ldc = (ld, M, ld) if inplace else (M, M, N)
    A = rng.uniform(-1, 1, K * lda)
    Bm = rng.uniform(-1, 1, N * ldb)
    C0 = A.copy() if inplace else rng.uniform(-1, 1, K * ldc)
    exp, den = common.tsmm_expected(M, N, K, A, lda, Bm, ldb, C0, ldc, 1.0, 0.5)
    mask = common.c_mask_tsmm(N, K, ldc)
    bound = common.tol(np.float64, M)
    Co = put(ref, C0, "float64")
    Ao = Co if inplace else put(ref, A, "float64")
    Bd = put(ref, Bm, "float64")
    handle.tsmm(M, N, K, Ao, lda, 1.0, Bd, ldb, 0.5, Co, ldc)
    ours = host(Co)
    assert _normwise(ours, exp, den, mask) <= bound
    variants = ["FIX3", "FIX_IP_GHOST"] if inplace else ["FIX3", "FIX_FB"]
    for variant in variants:
        Cr = put(ref, C0, "float64")
        Ar = Cr if inplace else put(ref, A, "float64")
        assert ref.tsmm(variant, M, N, K, Ar, lda, 1.0, Bd, ldb, 0.5, Cr, ldc, 2 * 152)
        ref_c = host(Cr)
        e_ref = _normwise(ref_c, exp, den, mask)
        assert e_ref <= bound, (variant, e_ref, bound)
        assert _normwise(ours, ref_c, den, mask) <= 2 * bound, variant
        # padding between rows untouched by both
        assert np.array_equal(ours[~mask], ref_c[~mask]), variant


@pytest.mark.parametrize("M", [1, 2, 4, 8, 16, 32, 64])
def test_c2_complex_in_place_against_fix_ip_ghost(ref, handle, M):
    """Complex FP64 in place (C2's complex in-place form), against the reference's complex-clean
    FIX_IP_GHOST kernel."""
    rng = np.random.default_rng(500 + M)
    K = 12007
    N = M
    A = common.uniform(rng, K * M, np.complex128)
    Bm = common.uniform(rng, N * M, np.complex128)
    exp, den = common.tsmm_expected(M, N, K, A, M, Bm, M, A.copy(), M, 1.0, 0.5)
    bound = common.tol(np.complex128, M)
    Co = put(ref, A, "complex128")
    Bd = put(ref, Bm, "complex128")
    handle.tsmm(M, N, K, Co, M, 1.0, Bd, M, 0.5, Co, M)
    ours = host(Co)
    Cr = put(ref, A, "complex128")
    assert ref.tsmm("FIX_IP_GHOST", M, N, K, Cr, M, 1.0, Bd, M, 0.5, Cr, M, 1, dtype="complex128")
    ref_c = host(Cr)
    mask = np.ones(K * M, dtype=bool)
    assert _normwise(ours, exp, den, mask) <= bound
    assert _normwise(ref_c, exp, den, mask) <= bound
    assert _normwise(ours, ref_c, den, mask) <= 2 * bound


def test_kat_double_double_against_specsmall_pseudoquad(ref, handle):
    """numeric_tests.cu:58-61: SPECSMALL<double, double> and SPECSMALL<double, PseudoQuad>, 1 x 1,
    blockCount 1000, N = 111113, against this library's native and dd methods."""
    a, b, d = common.kat()
    N = len(a)
    exact = d["exact_hi"]
    Ad, Bd = put(ref, a, "float64"), put(ref, b, "float64")
    out = {}
    for name in ("SPECSMALL", "SPECSMALL_PQ"):
        C = put(ref, np.zeros(1), "float64")
        assert ref.tsmttsm(name, 1, 1, N, Ad, 1, 1.0, Bd, 1, 0.0, C, 1, 1000)
        out[name] = float(host(C)[0])
    for acc in ("native", "dd"):
        C = put(ref, np.zeros(1), "float64")
        handle.tsmttsm(1, 1, N, Ad, 1, 1.0, Bd, 1, 0.0, C, 1, acc=acc)
        out[acc] = float(host(C)[0])
    err = {k: abs(v - exact) for k, v in out.items()}
    print("KAT exact", exact, "results", out, "errors", err)
    scale = float(np.abs(a) @ np.abs(b))
    # double-double keeps the small terms that FP64 loses next to the 2^124 products, on both sides
    assert err["SPECSMALL_PQ"] < 0.5 * err["SPECSMALL"], err
    assert err["dd"] < 0.5 * err["native"], err
    # both within the FP64 normwise bound of the exact value
    for k in ("SPECSMALL_PQ", "dd"):
        assert err[k] / scale <= common.tol(np.float64, N), (k, err[k])
    # the two double-double results agree to within the larger of their own errors
    assert abs(out["dd"] - out["SPECSMALL_PQ"]) <= max(err["dd"], err["SPECSMALL_PQ"]) + 4 * np.spacing(exact), out
