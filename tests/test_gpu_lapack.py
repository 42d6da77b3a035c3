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
