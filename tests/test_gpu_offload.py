"""GPU tests of the tile-offload interface (ooc_offload.h), against numpy/scipy in FP64.

Each reference call (ooc_offload.h:28-64) is checked on small ragged shapes: copies are
exact, BLAS/LAPACK results agree to RTOL relative to the operands' scale.
"""
import itertools

import numpy as np
import pytest
import scipy.linalg as sla

pytestmark = pytest.mark.gpu

RTOL = 1e-13


@pytest.fixture(scope="module")
def off(ooc, handle):
    from oocdag_gb300 import offload

    assert offload.init(0) == 0
    yield offload
    offload.destroy()


def _put(off, M):
    M = np.asfortranarray(M)
    p = off.Alloc(M.nbytes, 0)
    assert p != 0
    off.dSetMatrix(M.shape[0], M.shape[1], M, M.shape[0], p, M.shape[0], 0)
    return p


def _get(off, p, rows, cols):
    out = np.asfortranarray(np.zeros((rows, cols)))
    off.dGetMatrix(rows, cols, p, rows, out, rows, 0)
    return out


def test_copies_round_trip(off):
    rng = np.random.default_rng(0)
    A = np.asfortranarray(rng.standard_normal((37, 23)))
    p = _put(off, A)
    np.testing.assert_array_equal(_get(off, p, 37, 23), A)
    # strided vectors: every 3rd element in, every 2nd element on the device
    x = rng.standard_normal(60)
    d = off.Alloc(8 * 40, 1)
    off.dSetVector(20, x, 3, d, 2, 1)
    y = np.zeros(60)
    off.dGetVector(20, d, 2, y, 3, 1)
    np.testing.assert_array_equal(y[::3], x[::3])
    # device dcopy
    d2 = off.Alloc(8 * 20, 1)
    off.dcopy(20, d, 2, d2, 1, 1)
    z = np.zeros(20)
    off.dGetVector(20, d2, 1, z, 1, 1)
    np.testing.assert_array_equal(z, x[::3])
    # triangular copies move only the trapezoid
    for uplo in "LU":
        T = np.asfortranarray(rng.standard_normal((9, 6)))
        q = off.Alloc(T.nbytes, 2)
        zero = np.asfortranarray(np.zeros((9, 6)))
        off.dSetMatrix(9, 6, zero, 9, q, 9, 2)
        off.dtrSetMatrix(uplo, 9, 6, T, 9, q, 9, 2)
        back = _get(off, q, 9, 6)
        mask = np.tril(np.ones((9, 6), bool)) if uplo == "L" else np.triu(np.ones((9, 6), bool))
        np.testing.assert_array_equal(back[mask], T[mask])
        assert np.all(back[~mask] == 0)
        H = np.asfortranarray(np.full((9, 6), 5.0))
        off.dtrGetMatrix(uplo, 9, 6, q, 9, H, 9, 2)
        np.testing.assert_array_equal(H[mask], T[mask])
        assert np.all(H[~mask] == 5.0)
        off.Free(q, 2)
    for ptr in (p, d, d2):
        off.Free(ptr, 0)
    assert off.last_error() == 0


@pytest.mark.parametrize("ta,tb", list(itertools.product("NT", "NT")))
def test_dgemm(off, ta, tb):
    rng = np.random.default_rng(1)
    m, n, k = 70, 45, 33
    A = rng.standard_normal((m, k) if ta == "N" else (k, m))
    B = rng.standard_normal((k, n) if tb == "N" else (n, k))
    C = rng.standard_normal((m, n))
    alpha, beta = -1.5, 0.75
    want = alpha * (A if ta == "N" else A.T) @ (B if tb == "N" else B.T) + beta * C
    pa, pb, pc = _put(off, A), _put(off, B), _put(off, C)
    off.dgemm(ta, tb, m, n, k, alpha, pa, A.shape[0], pb, B.shape[0], beta, pc, m)
    got = _get(off, pc, m, n)
    assert np.abs(got - want).max() <= RTOL * np.abs(want).max() * k
    for p in (pa, pb, pc):
        off.Free(p)


@pytest.mark.parametrize("uplo,trans", list(itertools.product("LU", "NT")))
def test_dsyrk(off, uplo, trans):
    rng = np.random.default_rng(2)
    n, k = 67, 29
    A = rng.standard_normal((n, k) if trans == "N" else (k, n))
    C = rng.standard_normal((n, n))
    AA = A @ A.T if trans == "N" else A.T @ A
    want = -1.0 * AA + 1.0 * C
    pa, pc = _put(off, A), _put(off, C)
    off.dsyrk(uplo, trans, n, k, -1.0, pa, A.shape[0], 1.0, pc, n)
    got = _get(off, pc, n, n)
    tri = np.tril(np.ones((n, n), bool)) if uplo == "L" else np.triu(np.ones((n, n), bool))
    assert np.abs(got - want)[tri].max() <= RTOL * np.abs(want).max() * k
    np.testing.assert_array_equal(got[~tri], C[~tri])
    off.Free(pa)
    off.Free(pc)


@pytest.mark.parametrize("side,uplo,trans,diag", list(itertools.product("LR", "LU", "NT", "NU")))
def test_dtrsm(off, side, uplo, trans, diag):
    rng = np.random.default_rng(3)
    m, n = 53, 41
    kd = m if side == "L" else n
    T = rng.standard_normal((kd, kd)) * 0.1 + np.eye(kd) * 3.0  # well conditioned
    B = rng.standard_normal((m, n))
    alpha = 0.5
    Tt = np.tril(T) if uplo == "L" else np.triu(T)
    if diag == "U":
        np.fill_diagonal(Tt, 1.0)
    opT = Tt if trans == "N" else Tt.T
    want = alpha * (np.linalg.solve(opT, B) if side == "L" else np.linalg.solve(opT.T, B.T).T)
    pt, pb = _put(off, T), _put(off, B)
    off.dtrsm(side, uplo, trans, diag, m, n, alpha, pt, kd, pb, m)
    got = _get(off, pb, m, n)
    assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max(), (side, uplo, trans, diag)
    off.Free(pt)
    off.Free(pb)


@pytest.mark.parametrize("side,uplo,trans,diag", list(itertools.product("LR", "LU", "NT", "NU")))
def test_dtrsm_ill_conditioned_is_backward_stable(off, side, uplo, trans, diag):
    # A random triangle of order 200 has a condition number near 1e17: every form must
    # still leave a residual at FP64 rounding level (substitution, not an explicit inverse:
    # LAPACK's substitution gives 1e-21..4e-18 on these inputs, an explicit inverse up to 6e-17).
    rng = np.random.default_rng(17)
    m, n = 200, 130
    kd = m if side == "L" else n
    T = rng.standard_normal((kd, kd))
    np.fill_diagonal(T, rng.uniform(0.5, 1.5, kd) * np.sign(rng.standard_normal(kd)))
    B = rng.standard_normal((m, n))
    alpha = -1.5
    Tt = np.tril(T) if uplo == "L" else np.triu(T)
    if diag == "U":
        np.fill_diagonal(Tt, 1.0)
    opT = Tt if trans == "N" else Tt.T
    pt, pb = _put(off, T), _put(off, B)
    off.dtrsm(side, uplo, trans, diag, m, n, alpha, pt, kd, pb, m)
    X = _get(off, pb, m, n)
    R = opT @ X - alpha * B if side == "L" else X @ opT - alpha * B
    nrm = np.abs(opT).sum(1).max() * np.abs(X).max() + abs(alpha) * np.abs(B).max()
    assert np.abs(R).max() / nrm <= 2e-16, (side, uplo, trans, diag)
    off.Free(pt)
    off.Free(pb)


@pytest.mark.parametrize("uplo", "LU")
@pytest.mark.parametrize("n", [1, 63, 200])
def test_dpotrf(off, uplo, n):
    rng = np.random.default_rng(4)
    M = rng.standard_normal((n, n))
    A = M @ M.T / n + np.eye(n)
    pa = _put(off, A)
    assert off.dpotrf(uplo, n, pa, n) == 0
    got = _get(off, pa, n, n)
    L = np.linalg.cholesky(A)
    if uplo == "L":
        assert np.abs(np.tril(got) - L).max() <= 1e-12 * np.abs(L).max()
        np.testing.assert_array_equal(np.triu(got, 1), np.triu(A, 1))
    else:
        assert np.abs(np.triu(got) - L.T).max() <= 1e-12 * np.abs(L).max()
        np.testing.assert_array_equal(np.tril(got, -1), np.tril(A, -1))
    # not positive definite -> info = order of the failing minor
    B = A.copy()
    B[n // 2, n // 2] = -1.0
    pb = _put(off, B)
    assert off.dpotrf(uplo, n, pb, n) == n // 2 + 1
    off.Free(pa)
    off.Free(pb)


def test_argument_errors_reported(off):
    pa = off.Alloc(8 * 16)
    off.dgemm("X", "N", 4, 4, 4, 1.0, pa, 4, pa, 4, 0.0, pa, 4)
    assert off.last_error() == -1
    assert off.dpotrf("Q", 4, pa, 4) == -1
    off.Free(pa)
