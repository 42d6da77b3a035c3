"""ScaLAPACK-compatible entry points (1 x 1 grid) on the GPU, through the
C ABI as a ScaLAPACK caller would reach them: descriptors with MB as the
tile size, 1-based submatrix offsets inside larger local arrays.

Bar: pivots equal the oracle's (SLATE's getrf restated, nb = MB) on rows with
a clear pivot margin, and sit at IPIV(ia - 1 + r) offset by ia - 1; backward
error <= 3 eps64 (FP64) or the mixed solver's 3 n eps64; entries outside the
submatrix untouched; inverses and condition estimates as LAPACK's.
"""
import ctypes

import numpy as np
import pytest

from gpu_util import EPS, spd
from scalapack_util import call, desc, ip, pdgesv, ptr

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def L(slt):
    return ctypes.CDLL(slt.LIB_PATH)


def _berr(A, X, B):
    r = B - A @ X
    return np.abs(r).sum(0).max() / (A.shape[0] * np.abs(A).sum(0).max() * np.abs(X).sum(0).max())


def _check_pivots(orc, A, ipiv_lapack, nb):
    n = A.shape[0]
    oinfo, pt, po, oipiv, mg = orc.getrf(A.copy(order="F"), nb, min(16, nb), margins=True)
    robust = mg > 1 + 1e3 * n * EPS
    assert np.array_equal(ipiv_lapack[robust], oipiv[robust])


@pytest.mark.parametrize("n,mb", [(300, 64), (129, 32)])
def test_pdgesv_whole_matrix(orc, L, n, mb):
    A = orc.generate(2, 301, n, n)
    B = orc.generate(2, 302, n, 3)
    a, b = A.copy(order="F"), B.copy(order="F")
    piv = np.zeros(n, np.int32)
    info = pdgesv(L, n, 3, a, 1, 1, desc(n, n, mb, n), piv, b, 1, 1, desc(n, 3, mb, n))
    assert info == 0
    assert _berr(A, b, B) <= 3 * EPS
    _check_pivots(orc, A, piv.astype(np.int64), mb)


def test_pdgesv_submatrix(orc, L):
    """A(65:364, 65:364) inside a 400 x 400 local array with LLD 410, the
    right-hand sides B(33:332, 2:3) inside a 350 x 4 array."""
    M, lld, n, ia = 400, 410, 300, 65
    G = np.asfortranarray(orc.generate(2, 303, lld, M))
    H = np.asfortranarray(orc.generate(2, 304, 350, 4))
    A = G[ia - 1:ia - 1 + n, ia - 1:ia - 1 + n].copy()
    B = H[32:32 + n, 1:3].copy()
    g, h = G.copy(order="F"), H.copy(order="F")
    piv = np.full(M, -7, np.int32)
    info = pdgesv(L, n, 2, g, ia, ia, desc(M, M, 64, lld), piv, h, 33, 2, desc(350, 4, 64, 350))
    assert info == 0
    X = h[32:32 + n, 1:3]
    assert _berr(A, X, B) <= 3 * EPS
    # outside the submatrices nothing changed
    mask = np.ones_like(G, bool)
    mask[ia - 1:ia - 1 + n, ia - 1:ia - 1 + n] = False
    assert np.array_equal(g[mask], G[mask])
    hm = np.ones_like(H, bool)
    hm[32:32 + n, 1:3] = False
    assert np.array_equal(h[hm], H[hm])
    # IPIV(ia - 1 + r) = global row; untouched elsewhere
    assert (piv[:ia - 1] == -7).all() and (piv[ia - 1 + n:] == -7).all()
    _check_pivots(orc, A, piv[ia - 1:ia - 1 + n].astype(np.int64) - (ia - 1), 64)


def test_pdgetrf_pdgetrs(orc, L):
    n = 257
    A = orc.generate(2, 305, n, n)
    B = orc.generate(2, 306, n, 2)
    a = A.copy(order="F")
    piv = np.zeros(n, np.int32)
    da = desc(n, n, 64, n)
    assert call(L, "pdgetrf_", ip(n), ip(n), ptr(a), ip(1), ip(1), ptr(da), ptr(piv)) == 0
    _check_pivots(orc, A, piv.astype(np.int64), 64)
    for trans, op in ((b"N", A), (b"T", A.T)):
        b = B.copy(order="F")
        assert call(L, "pdgetrs_", trans, ip(n), ip(2), ptr(a), ip(1), ip(1), ptr(da), ptr(piv), ptr(b), ip(1), ip(1),
                    ptr(desc(n, 2, 64, n))) == 0
        assert _berr(np.asfortranarray(op), b, B) <= 3 * EPS


def test_pdgetrf_singular_info(orc, L):
    n = 100
    A = orc.generate(2, 307, n, n)
    A[:, 40] = 0.0
    a = A.copy(order="F")
    piv = np.zeros(n, np.int32)
    assert call(L, "pdgetrf_", ip(n), ip(n), ptr(a), ip(1), ip(1), ptr(desc(n, n, 32, n)), ptr(piv)) == 41


@pytest.mark.parametrize("uplo", [b"L", b"U"])
def test_pdposv_pdpotrf_pdpotrs(orc, L, uplo):
    n = 300
    A = spd(orc, n, 308)
    B = orc.generate(2, 309, n, 3)
    da, db = desc(n, n, 64, n), desc(n, 3, 64, n)
    a, b = A.copy(order="F"), B.copy(order="F")
    assert call(L, "pdposv_", uplo, ip(n), ip(3), ptr(a), ip(1), ip(1), ptr(da), ptr(b), ip(1), ip(1), ptr(db)) == 0
    assert _berr(A, b, B) <= 3 * EPS
    a, b = A.copy(order="F"), B.copy(order="F")
    assert call(L, "pdpotrf_", uplo, ip(n), ptr(a), ip(1), ip(1), ptr(da)) == 0
    C = np.linalg.cholesky(A)
    F = np.tril(a) if uplo == b"L" else np.triu(a).T
    np.testing.assert_allclose(F, C, rtol=0, atol=1e-12 * np.abs(A).max())
    assert call(L, "pdpotrs_", uplo, ip(n), ip(3), ptr(a), ip(1), ip(1), ptr(da), ptr(b), ip(1), ip(1), ptr(db)) == 0
    assert _berr(A, b, B) <= 3 * EPS


def test_pdpotrf_not_spd(orc, L):
    n = 90
    A = spd(orc, n, 310)
    A[50, 50] = -1.0
    a = A.copy(order="F")
    assert call(L, "pdpotrf_", b"L", ip(n), ptr(a), ip(1), ip(1), ptr(desc(n, n, 32, n))) == orc.potrf(A.copy(order="F"), 32)


def test_pdsgesv(orc, L):
    n = 400
    A = orc.generate(2, 311, n, n)
    B = orc.generate(2, 312, n, 2)
    a, b = A.copy(order="F"), B.copy(order="F")
    x = np.zeros((n, 2), order="F")
    piv = np.zeros(n, np.int32)
    it = ctypes.c_int(-99)
    d, d2 = desc(n, n, 128, n), desc(n, 2, 128, n)
    info = call(L, "pdsgesv_", ip(n), ip(2), ptr(a), ip(1), ip(1), ptr(d), ptr(piv), ptr(b), ip(1), ip(1), ptr(d2),
                ptr(x), ip(1), ip(1), ptr(d2), ctypes.byref(it))
    assert info == 0 and it.value >= 0
    assert _berr(A, x, B) <= 3 * n * EPS


def test_pdgetri_pdpotri(orc, L):
    n = 200
    A = orc.generate(2, 313, n, n)
    a = A.copy(order="F")
    piv = np.zeros(n, np.int32)
    d = desc(n, n, 64, n)
    assert call(L, "pdgetrf_", ip(n), ip(n), ptr(a), ip(1), ip(1), ptr(d), ptr(piv)) == 0
    work = np.zeros(1)
    iwork = np.zeros(1, np.int32)
    assert call(L, "pdgetri_", ip(n), ptr(a), ip(1), ip(1), ptr(d), ptr(piv), ptr(work), ip(1), ptr(iwork),
                ip(1)) == 0
    Ai = np.linalg.inv(A)
    assert np.abs(a - Ai).max() <= 1e-10 * np.abs(Ai).max()
    S = spd(orc, n, 314)
    s = S.copy(order="F")
    assert call(L, "pdpotrf_", b"L", ip(n), ptr(s), ip(1), ip(1), ptr(d)) == 0
    assert call(L, "pdpotri_", b"L", ip(n), ptr(s), ip(1), ip(1), ptr(d)) == 0
    Si = np.linalg.inv(S)
    assert np.abs(np.tril(s) - np.tril(Si)).max() <= 1e-10 * np.abs(Si).max()


def test_pdgecon_pdpocon(orc, L):
    import scipy.linalg.lapack as lp
    n = 250
    A = orc.generate(2, 315, n, n)
    anorm = np.abs(A).sum(0).max()
    a = A.copy(order="F")
    piv = np.zeros(n, np.int32)
    d = desc(n, n, 64, n)
    assert call(L, "pdgetrf_", ip(n), ip(n), ptr(a), ip(1), ip(1), ptr(d), ptr(piv)) == 0
    rc = ctypes.c_double(0.0)
    work = np.zeros(1)
    iwork = np.zeros(1, np.int32)
    assert call(L, "pdgecon_", b"1", ip(n), ptr(a), ip(1), ip(1), ptr(d), ctypes.byref(ctypes.c_double(anorm)),
                ctypes.byref(rc), ptr(work), ip(1), ptr(iwork), ip(1)) == 0
    lu, _, _ = lp.dgetrf(A)
    ref, _ = lp.dgecon(lu, anorm, norm="1")
    assert abs(rc.value - ref) <= 0.01 * ref
    S = spd(orc, n, 316)
    snorm = np.abs(S).sum(0).max()
    s = S.copy(order="F")
    assert call(L, "pdpotrf_", b"L", ip(n), ptr(s), ip(1), ip(1), ptr(d)) == 0
    assert call(L, "pdpocon_", b"L", ip(n), ptr(s), ip(1), ip(1), ptr(d), ctypes.byref(ctypes.c_double(snorm)),
                ctypes.byref(rc), ptr(work), ip(1), ptr(iwork), ip(1)) == 0
    c, _ = lp.dpotrf(S, lower=1)
    ref, _ = lp.dpocon(c, snorm, uplo="L")
    assert abs(rc.value - ref) <= 0.01 * ref


def test_psgesv(orc, L):
    n = 200
    A = orc.generate(2, 317, n, n).astype(np.float32)
    B = orc.generate(2, 318, n, 2).astype(np.float32)
    a, b = np.asfortranarray(A.copy()), np.asfortranarray(B.copy())
    piv = np.zeros(n, np.int32)
    info = call(L, "psgesv_", ip(n), ip(2), ptr(a), ip(1), ip(1), ptr(desc(n, n, 32, n)), ptr(piv), ptr(b), ip(1),
                ip(1), ptr(desc(n, 2, 32, n)))
    assert info == 0
    r = B.astype(np.float64) - A.astype(np.float64) @ b.astype(np.float64)
    e = np.abs(r).sum(0).max() / (n * np.abs(A).sum(0).max() * np.abs(b).sum(0).max())
    assert e <= 3 * np.finfo(np.float32).eps
