"""The LAPACK-compatible host entry points (slate_dgesv & co.) against LAPACK."""
import numpy as np
import pytest
import scipy.linalg as sl

from gpu_util import EPS, spd

pytestmark = pytest.mark.gpu


def test_slate_dgesv(orc, slt):
    n, nrhs = 900, 2
    A = orc.generate(2, 51, n, n)
    B = orc.generate(2, 52, n, nrhs)
    a, b = A.copy(order="F"), B.copy(order="F")
    info, ipiv = slt.lapack.dgesv(a, b)
    assert info == 0
    lu, piv = sl.lu_factor(A)
    assert np.array_equal(ipiv - 1, piv)
    assert orc.backward_error(A, b, B) <= 3 * EPS


def test_slate_dgetrf_dgetrs(orc, slt):
    n = 513
    A = orc.generate(2, 61, n, n)
    a = A.copy(order="F")
    info, ipiv = slt.lapack.dgetrf(a)
    assert info == 0
    B = orc.generate(2, 62, n, 3)
    b = B.copy(order="F")
    assert slt.lapack.dgetrs(a, ipiv, b) == 0
    assert orc.backward_error(A, b, B) <= 3 * EPS
    # factors from LAPACK itself solve through slate_dgetrs too
    lu, piv = sl.lu_factor(A)
    b = B.copy(order="F")
    assert slt.lapack.dgetrs(np.asfortranarray(lu), (piv + 1).astype(np.int32), b) == 0
    assert orc.backward_error(A, b, B) <= 3 * EPS


def test_slate_dsgesv(orc, slt):
    n = 700
    A = orc.generate(2, 71, n, n)
    B = orc.generate(2, 72, n, 2)
    x = np.zeros_like(B, order="F")
    info, it, ipiv = slt.lapack.dsgesv(A.copy(order="F"), B.copy(order="F"), x)
    assert info == 0 and it >= 0
    assert orc.backward_error(A, x, B) <= 3 * n * EPS


@pytest.mark.parametrize("uplo", ["L", "U"])
def test_slate_dposv_dpotrf(orc, slt, uplo):
    n = 600
    A = spd(orc, n, 81)
    B = orc.generate(2, 82, n, 2)
    a, b = A.copy(order="F"), B.copy(order="F")
    assert slt.lapack.dposv(uplo, a, b) == 0
    assert orc.backward_error(A, b, B) <= 3 * EPS
    a = A.copy(order="F")
    assert slt.lapack.dpotrf(uplo, a) == 0
    c = sl.cholesky(A, lower=(uplo == "L"))
    tri = np.tril if uplo == "L" else np.triu
    np.testing.assert_allclose(tri(a), c, atol=1e-12)


def _call_chol(slt, name, uplo, A, lda, B=None, X=None):
    """slate_dposv / slate_dpotrf / slate_dsposv on Fortran arrays with a
    leading dimension above n (the extra rows hold NaN)."""
    import ctypes
    c = ctypes.c_int
    n = A.shape[0]
    a = np.full((lda, n), np.nan, order="F")
    a[:n] = A
    info, it = c(0), c(0)
    p = lambda m: m.ctypes.data_as(ctypes.c_void_p)
    L = slt.lib()
    if name == "dpotrf":
        L.slate_dpotrf(ctypes.c_char_p(uplo.encode()), ctypes.byref(c(n)), p(a), ctypes.byref(c(lda)),
                       ctypes.byref(info))
    elif name == "dposv":
        L.slate_dposv(ctypes.c_char_p(uplo.encode()), ctypes.byref(c(n)), ctypes.byref(c(B.shape[1])), p(a),
                      ctypes.byref(c(lda)), p(B), ctypes.byref(c(n)), ctypes.byref(info))
    else:
        L.slate_dsposv(ctypes.c_char_p(uplo.encode()), ctypes.byref(c(n)), ctypes.byref(c(B.shape[1])), p(a),
                       ctypes.byref(c(lda)), p(B), ctypes.byref(c(n)), p(X), ctypes.byref(c(n)), None, None,
                       ctypes.byref(it), ctypes.byref(info))
    return info.value, it.value, a


@pytest.mark.parametrize("uplo", ["L", "U"])
def test_cholesky_entry_points_read_only_their_triangle(orc, slt, uplo):
    """slate_dpotrf / dposv / dsposv copy only the referenced triangle: the
    other one holds NaN on entry (not read) and is unchanged on exit, as are
    the rows beyond n of a leading dimension above n; n is off the 512-column
    blocks of the copies."""
    n, nrhs, lda = 1100, 3, 1107
    A = spd(orc, n, 83)
    other = np.triu_indices(n, 1) if uplo == "L" else np.tril_indices(n, -1)
    Ain = A.copy(order="F")
    Ain[other] = np.nan
    tri = np.tril if uplo == "L" else np.triu
    # dpotrf: the factor in the referenced triangle
    info, _, a = _call_chol(slt, "dpotrf", uplo, Ain, lda)
    assert info == 0
    np.testing.assert_allclose(tri(np.nan_to_num(a[:n])), sl.cholesky(A, lower=(uplo == "L")), atol=1e-12)
    assert np.all(np.isnan(a[:n][other])) and np.all(np.isnan(a[n:]))
    # dposv: the solution, the factor in A
    B = orc.generate(2, 84, n, nrhs)
    b = B.copy(order="F")
    info, _, a = _call_chol(slt, "dposv", uplo, Ain, lda, B=b)
    assert info == 0
    assert orc.backward_error(A, b, B) <= 3 * EPS
    assert np.all(np.isnan(a[:n][other])) and np.all(np.isnan(a[n:]))
    # dsposv: refinement converged, A unchanged
    x = np.zeros((n, nrhs), order="F")
    info, it, a = _call_chol(slt, "dsposv", uplo, Ain, lda, B=B.copy(order="F"), X=x)
    assert info == 0 and it >= 0
    assert orc.backward_error(A, x, B) <= 3 * n * EPS
    assert np.array_equal(a[:n][~np.isnan(Ain)], Ain[~np.isnan(Ain)])
    assert np.all(np.isnan(a[:n][other])) and np.all(np.isnan(a[n:]))
    # dsposv with the FP64 fallback (kappa beyond FP32): A holds the FP64 factor
    S = orc.generate_sigma(n, 1e14, "geo", True, 7)
    Sin = S.copy(order="F")
    Sin[other] = np.nan
    x = np.zeros((n, nrhs), order="F")
    info, it, a = _call_chol(slt, "dsposv", uplo, Sin, lda, B=B.copy(order="F"), X=x)
    assert info == 0 and it < 0
    assert orc.backward_error(S, x, B) <= 3 * n * EPS
    F = tri(np.nan_to_num(a[:n]))
    R = F @ F.T if uplo == "L" else F.T @ F              # the factor reproduces S
    assert np.abs(R - S).max() <= 8 * n * EPS * np.abs(S).max()
    assert np.all(np.isnan(a[:n][other])) and np.all(np.isnan(a[n:]))


@pytest.mark.parametrize("refine", ["gmres", "ir"])
@pytest.mark.parametrize("stream", ["1", "2", "0"])
def test_dsposv_streamed_lower_triangle(orc, slt, monkeypatch, refine, stream):
    """slate_dsposv with an FP16 factor: the lower triangle of A arrives by
    512-column blocks on a copy stream while the left-looking factor consumes
    it (SLATE_LAPACK_STREAM=1, the default; =2 whole block columns, here 2-D
    copies since lda > n) or is copied before the solve (=0); same solution
    quality, A unchanged, NaN above the diagonal never read; n off the block
    size, lda above n."""
    monkeypatch.setenv("SLATE_LAPACK_FACTOR_PRECISION", "fp16")
    monkeypatch.setenv("SLATE_LAPACK_REFINE", refine)
    monkeypatch.setenv("SLATE_LAPACK_STREAM", stream)
    monkeypatch.setenv("SLT_POTRF_LL", "1")
    n, nrhs, lda = 3000, 4, 3011
    A = spd(orc, n, 85)
    B = orc.generate(2, 86, n, nrhs)
    Ain = A.copy(order="F")
    Ain[np.triu_indices(n, 1)] = np.nan
    x = np.zeros((n, nrhs), order="F")
    info, it, a = _call_chol(slt, "dsposv", "L", Ain, lda, B=B.copy(order="F"), X=x)
    assert info == 0 and it >= 0, (info, it)
    assert orc.backward_error(A, x, B) <= 3 * n * EPS
    keep = ~np.isnan(Ain)
    assert np.array_equal(a[:n][keep], Ain[keep]) and np.all(np.isnan(a[n:]))
