"""GPU test of include/skinny.hpp: a C++ driver written like the reference's test harness calls the
reference-spelled launchers (GENV5::tsmttsm<double, 8, 8>, SPECSMALL::tsmttsm<double, PseudoQuad,
...>, tsmm_fix3<...>, tsmm_var1<...>) on integer data; every result is compared exactly with
numpy, and a launcher whose template (M, N) differs from the runtime one must return false."""
import os
import shutil
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def data(K, M, N, tsmm):
    i = np.arange(K * M)
    A = ((i * 7 + 3) % 11 - 5).astype(np.float64)
    j = np.arange(M * N if tsmm else K * N)
    B = ((j * 5 + 1) % 9 - 4).astype(np.float64)
    c = np.arange(K * N if tsmm else M * N)
    C = (c % 5 - 2).astype(np.float64)
    return A, B, C


def expected_sum(K, M, N, tsmm):
    A, B, C = data(K, M, N, tsmm)
    if tsmm:
        out = A.reshape(K, M) @ B.reshape(N, M).T + 0.5 * C.reshape(K, N)
    else:
        out = (A.reshape(K, M).T @ B.reshape(K, N)).T + 0.5 * C.reshape(N, M)
    return float(out.sum())


def test_reference_spelled_launchers(skinny_lib, tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ missing")
    build = os.path.join(ROOT, "skinny_matmul_gb300", "_build")
    exe = str(tmp_path / "shim_driver")
    cmd = [gxx, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), "-I", "/usr/local/cuda/include",
           os.path.join(ROOT, "tests", "cpp", "shim_driver.cpp"), "-o", exe, "-L", build, "-lskinny",
           "-Wl,-rpath," + build, "-L", "/usr/local/cuda/lib64", "-lcudart", "-Wl,-rpath,/usr/local/cuda/lib64"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    got = {ln.split()[0]: (int(ln.split()[1]), float(ln.split()[2])) for ln in r.stdout.strip().splitlines()}
    K = 10000
    assert got["GENV5_8x8"] == (1, expected_sum(K, 8, 8, False))
    assert got["SPECSMALL_PQ_4x4"] == (1, expected_sum(K, 4, 4, False))
    assert got["GENV3_GLOBAL_2x3"] == (1, expected_sum(K, 2, 3, False))
    assert got["FIX3_4x4"] == (1, expected_sum(K, 4, 4, True))
    assert got["VAR1_3x5"] == (1, expected_sum(K, 3, 5, True))
    # template (8, 8) with runtime (4, 4): not launched, C untouched
    _, _, C0 = data(K, 4, 4, False)
    assert got["MISMATCH"] == (0, float(C0.sum()))
