"""CPU tests of the host double-double SVQB (skinny_svqb_host_dd, the reference's high-precision
study svqb/svqb.cu:132-182): it needs no GPU, so these run in the CPU suite.

Bars:
  * condition 1e3: Q equals the oracle's one-pass SVQB (oracle/svqb.py, exact Gram, FP64
    eigensolve) up to column signs within kappa^2 * 8 sqrt(K) u, and ||Q^T Q - I||_F <= 1e-14;
  * condition 1e8: ||Q^T Q - I||_F <= 1e-14 where a one-pass FP64 SVQB reaches ~1e-2..1 (the
    study's point: the eigensolve's precision, not the Gram's, limits a single pass), and Q spans
    X (||X - Q Q^T X||_F / ||X||_F <= 1e-12);
  * the reported orthogonality error equals the oracle's (exact Gram of the rounded Q);
  * the result does not depend on the number of host threads beyond the last bit;
  * bad arguments are refused before any work.
"""
import math

import numpy as np
import pytest

from oracle import svqb as OS


@pytest.fixture(scope="module")
def api(skinny_lib):
    from skinny_matmul_gb300 import api as A
    return A


def _sign_align(Q, R, K, M):
    Q2, R2 = Q.reshape(K, M), R.reshape(K, M)
    s = np.sign(np.sum(Q2 * R2, axis=0))
    return Q2 * s[None, :], R2


def test_well_conditioned_matches_oracle(api):
    K, M, cond = 4096, 16, 1e3
    X = OS.make_x(K, M, cond, seed=11)
    Q, err = api.svqb_host_dd(X, K, M, threads=4)
    Qr = OS.svqb(X, K, M, "exact")
    Qa, Ra = _sign_align(Q, Qr, K, M)
    rel = np.linalg.norm(Qa - Ra) / np.linalg.norm(Ra)
    assert rel <= cond ** 2 * 8 * math.sqrt(K) * 2.0 ** -53, rel
    assert err <= 1e-14, err
    assert abs(err - OS.orth_error(Q, K, M)) <= 1e-16 + 1e-6 * err


@pytest.mark.parametrize("M", [8, 32])
def test_ill_conditioned_stays_orthogonal(api, M):
    K, cond = 8192, 1e8
    X = OS.make_x(K, M, cond, seed=20 + M)
    Q, err = api.svqb_host_dd(X, K, M)
    assert err <= 1e-14, err
    fp64 = OS.orth_error(OS.svqb(X, K, M, "exact"), K, M)
    assert fp64 > 1e3 * err, (fp64, err)  # a one-pass FP64 SVQB is far from orthogonal here
    X2, Q2 = X.reshape(K, M), Q.reshape(K, M)
    resid = np.linalg.norm(X2 - Q2 @ (Q2.T @ X2)) / np.linalg.norm(X2)
    assert resid <= 1e-12, resid


def test_thread_count_changes_only_the_last_bit(api):
    K, M = 3000, 12
    X = OS.make_x(K, M, 1e4, seed=5)
    Q1, _ = api.svqb_host_dd(X, K, M, threads=1, orth_err=False)
    Q7, _ = api.svqb_host_dd(X, K, M, threads=7, orth_err=False)
    assert np.max(np.abs(Q1 - Q7)) <= 4 * np.spacing(np.max(np.abs(Q1)))


def test_zero_column_gets_zero_scaling(api):
    """A zero column has S_ii = 0 <= eps: its scaling is 0, as in the reference."""
    K, M = 500, 4
    X = OS.make_x(K, M, 10.0, seed=3).reshape(K, M)
    X[:, 2] = 0.0
    Q, _ = api.svqb_host_dd(X.ravel(), K, M, orth_err=False)
    assert np.all(np.isfinite(Q))


def test_bad_arguments(api, skinny_lib):
    import ctypes
    buf = np.zeros(16)
    assert skinny_lib.skinny_svqb_host_dd(None, buf.ctypes.data, 4, 4, 1, None) != 0
    assert skinny_lib.skinny_svqb_host_dd(buf.ctypes.data, buf.ctypes.data, 4, 0, 1, None) != 0
    assert skinny_lib.skinny_svqb_host_dd(buf.ctypes.data, buf.ctypes.data, -1, 4, 1, ctypes.c_void_p()) != 0
