"""The oracle's restated algorithms against LAPACK (scipy) and known answers.

SLATE ships no golden vectors for getrf/potrf/gesv, so the restatement is
cross-checked against LAPACK: identical pivots where the pivot choice is
robust, tiny factor differences, and the tester's residual check.
"""
import numpy as np
import pytest
import scipy.linalg as sl

EPS = np.finfo(np.float64).eps


@pytest.mark.parametrize("n,nb,ib", [(1, 4, 2), (7, 4, 2), (64, 16, 4), (100, 32, 16), (257, 64, 16)])
def test_getrf_matches_lapack(orc, n, nb, ib):
    A = orc.generate(2, 1000 + n, n, n)
    A0 = A.copy(order="F")
    info, pt, po, ipiv, mg = orc.getrf(A, nb, ib, margins=True)
    assert info == 0
    lu, piv = sl.lu_factor(A0)
    robust = mg > 1 + 1e3 * n * EPS
    assert np.array_equal((ipiv - 1)[robust], piv[robust])
    assert np.abs(lu - A).max() < 1e-10 * max(1.0, np.abs(lu).max())


def test_getrf_rectangular(orc):
    for m, n in ((50, 30), (30, 50)):
        A = orc.generate(2, 5, m, n)
        A0 = A.copy(order="F")
        info, pt, po, ipiv, _ = orc.getrf(A, 16, 4)
        lu, piv = sl.lu_factor(A0)
        assert info == 0
        assert np.array_equal(ipiv - 1, piv)
        assert np.abs(lu - A).max() < 1e-12


def test_gesv_backward_error(orc):
    n, nb = 300, 64
    A = orc.generate(2, 1, n, n)
    A0 = A.copy(order="F")
    B = orc.generate(2, 2, n, 3)
    B0 = B.copy(order="F")
    info, pt, po = orc.gesv(A, B, nb)
    assert info == 0
    assert orc.backward_error(A0, B, B0) <= 3 * EPS


def test_known_answers(orc):
    # identity: no interchanges, L = U = I
    A = orc.generate_kind("identity", 10, 10)
    info, pt, po, ipiv, _ = orc.getrf(A, 4, 2)
    assert info == 0 and np.array_equal(ipiv, np.arange(1, 11))
    assert np.array_equal(A, np.eye(10))
    # ones: rank one, U(2,2) is the first exact zero
    A = orc.generate_kind("ones", 8, 8)
    info, *_ = orc.getrf(A, 4, 2)
    assert info == 2
    # zeros: the first pivot is zero
    A = orc.generate_kind("zeros", 5, 5)
    info, *_ = orc.getrf(A, 4, 2)
    assert info == 1
    # minij is SPD with L = lower ones
    A = orc.generate_kind("minij", 12, 12)
    assert orc.potrf(A, 4) == 0
    np.testing.assert_allclose(np.tril(A), np.tril(np.ones((12, 12))), atol=1e-14)


def test_tie_break_follows_panel_threads(orc):
    # column 0 = [1, 3, 3, 3]: exact ties off the diagonal.  One panel thread
    # scans rows in order and keeps the first; with 2 threads over tiles of 1
    # row, thread 0 (rows 0, 2) wins the tie over thread 1 (rows 1, 3).
    A = np.asfortranarray(np.array([[1., 0, 0, 0], [3, 1, 0, 0], [3, 0, 1, 0], [3, 0, 0, 1]]))
    info, pt, po, ipiv, _ = orc.getrf(A.copy(order="F"), 1, 1, panel_threads=1)
    assert ipiv[0] == 2
    info, pt, po, ipiv, _ = orc.getrf(A.copy(order="F"), 1, 1, panel_threads=2)
    assert ipiv[0] == 3
    # a tie with the diagonal keeps the diagonal (pivot threshold rule)
    B = np.asfortranarray(np.array([[2., 1], [-2, 1]]))
    info, pt, po, ipiv, _ = orc.getrf(B, 2, 1)
    assert ipiv[0] == 1


def test_potrf_potrs(orc):
    n, nb = 200, 64
    G = orc.generate(3, 3, n, n)
    S = np.asfortranarray(G @ G.T / n + np.eye(n))
    S0 = S.copy(order="F")
    assert orc.potrf(S, nb) == 0
    np.testing.assert_allclose(np.tril(S), np.linalg.cholesky(S0), atol=1e-13)
    B = orc.generate(2, 4, n, 4)
    B0 = B.copy(order="F")
    orc.potrs(S, B, nb)
    assert orc.backward_error(S0, B, B0) <= 3 * EPS
    # not positive definite
    S1 = S0.copy(order="F")
    S1[50, 50] = -1.0
    assert orc.potrf(S1, nb) == 51


@pytest.mark.parametrize("fn", ["gesv_mixed", "gesv_mixed_gmres", "posv_mixed", "posv_mixed_gmres"])
def test_mixed_drivers(orc, fn):
    n, nb = 256, 64
    if fn.startswith("posv"):
        G = orc.generate(3, 11, n, n)
        A = np.asfortranarray(G @ G.T / n + np.eye(n))
    else:
        A = orc.generate(2, 12, n, n)
    A0 = A.copy(order="F")
    nrhs = 1 if "gmres" in fn else 3
    B = orc.generate(2, 13, n, nrhs)
    r = getattr(orc, fn)(A, B.copy(order="F") if nrhs > 1 else B[:, 0].copy(), nb)
    info, X, it = r[0], r[1], r[2]
    assert info == 0 and it >= 0
    assert orc.backward_error(A0, X, B, sym_lower=fn.startswith("posv")) <= 3 * n * EPS
    # forced non-convergence: iter = -(itermax+1) and the FP64 fallback solves
    A = A0.copy(order="F")
    r = getattr(orc, fn)(A, B.copy(order="F") if nrhs > 1 else B[:, 0].copy(), nb, itermax=0)
    assert r[2] == -1 and r[0] == 0
    assert orc.backward_error(A0, r[1], B, sym_lower=fn.startswith("posv")) <= 3 * EPS * 10


def test_mixed_singular_reports_info(orc):
    n = 64
    A = orc.generate(2, 3, n, n)
    A[:, 5] = 0.0
    B = orc.generate(2, 4, n, 1)
    info, X, it, _, _ = orc.gesv_mixed(A, B, 16)
    assert it == -3 and info > 0
