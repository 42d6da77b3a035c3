"""SLATE's C API (opaque handles, lu_* / chol_*) on the GPU, host and device data.

Bar: the same results as the library's own drivers (bit-identical factors
for the same inputs and tile size) and FP64 backward error <= 3 eps64;
SLATE's info on a singular / indefinite matrix.
"""
import ctypes

import numpy as np
import pytest

from gpu_util import EPS, berr, spd, to_dev, to_host

pytestmark = pytest.mark.gpu

vp, i64 = ctypes.c_void_p, ctypes.c_int64


def _api(slt):
    L = slt.lib()
    for name in ("slate_Matrix_create_fromScaLAPACK_r64",):
        getattr(L, name).restype = vp
        getattr(L, name).argtypes = [i64, i64, vp, i64, i64, i64, ctypes.c_int, ctypes.c_int, ctypes.c_ssize_t]
    L.slate_HermitianMatrix_create_fromScaLAPACK_r64.restype = vp
    L.slate_HermitianMatrix_create_fromScaLAPACK_r64.argtypes = [ctypes.c_char, i64, vp, i64, i64, ctypes.c_int,
                                                                 ctypes.c_int, ctypes.c_ssize_t]
    for name in ("slate_Options_create", "slate_Pivots_create"):
        getattr(L, name).restype = vp
    for name in ("slate_lu_solve_r64", "slate_chol_solve_r64", "slate_chol_solve_using_factor_r64"):
        getattr(L, name).argtypes = [vp, vp, vp]
    L.slate_lu_factor_r64.argtypes = [vp, vp, vp]
    L.slate_lu_solve_using_factor_r64.argtypes = [vp, vp, vp, vp]
    L.slate_chol_factor_r64.argtypes = [vp, vp]
    L.slate_gb300_last_info.restype = i64
    for name in ("slate_Matrix_destroy_r64", "slate_HermitianMatrix_destroy_r64", "slate_Options_destroy",
                 "slate_Pivots_destroy"):
        getattr(L, name).argtypes = [vp]
    L.slate_Options_set_BlockSize.argtypes = [vp, i64]
    return L


def _mat(L, arr_ptr, m, n, ld, nb):
    return L.slate_Matrix_create_fromScaLAPACK_r64(m, n, arr_ptr, ld, nb, nb, 1, 1, 0)


@pytest.mark.parametrize("where", ["host", "device"])
def test_c_api_lu(orc, slt, where):
    import torch
    L = _api(slt)
    n, nrhs, nb = 300, 3, 64
    A = orc.generate(2, 71, n, n)
    B = orc.generate(2, 72, n, nrhs)
    opts = L.slate_Options_create()
    # reference: the library's gesv on the device
    dA0, dB0 = to_dev(A), to_dev(B)
    slt.gesv(dA0, dB0, slt.Options(nb=nb))
    torch.cuda.synchronize()
    if where == "host":
        a, b = A.copy(order="F"), B.copy(order="F")
        ha, hb = _mat(L, a.ctypes.data, n, n, n, nb), _mat(L, b.ctypes.data, n, nrhs, n, nb)
    else:
        da, db = to_dev(A), to_dev(B)
        ha, hb = _mat(L, da.data_ptr(), n, n, n, nb), _mat(L, db.data_ptr(), n, nrhs, n, nb)
    L.slate_lu_solve_r64(ha, hb, opts)
    torch.cuda.synchronize()
    assert L.slate_gb300_last_status() == 0 and L.slate_gb300_last_info() == 0
    X = b if where == "host" else to_host(db)
    LU = a if where == "host" else to_host(da)
    assert np.array_equal(X, to_host(dB0)) and np.array_equal(LU, to_host(dA0))
    assert berr(orc, A, X, B) <= 3 * EPS
    # factor, then solve with the recorded pivots
    a2, b2 = A.copy(order="F"), B.copy(order="F")
    h2, hb2 = _mat(L, a2.ctypes.data, n, n, n, nb), _mat(L, b2.ctypes.data, n, nrhs, n, nb)
    piv = L.slate_Pivots_create()
    L.slate_lu_factor_r64(h2, piv, opts)
    L.slate_lu_solve_using_factor_r64(h2, piv, hb2, opts)
    assert L.slate_gb300_last_status() == 0
    assert np.array_equal(b2, X)
    for h in (ha, hb, h2, hb2):
        L.slate_Matrix_destroy_r64(h)
    L.slate_Pivots_destroy(piv)
    L.slate_Options_destroy(opts)


@pytest.mark.parametrize("uplo", [b"L", b"U"])
@pytest.mark.parametrize("where", ["host", "device"])
def test_c_api_chol(orc, slt, uplo, where):
    import torch
    L = _api(slt)
    n, nrhs, nb = 260, 2, 64
    A = spd(orc, n, 73)
    B = orc.generate(2, 74, n, nrhs)
    # store only the referenced triangle; the other one holds a marker value
    Ah = np.where(np.tril(np.ones((n, n))) if uplo == b"L" else np.triu(np.ones((n, n))), A, 7.0)
    Ah = np.asfortranarray(Ah)
    opts = L.slate_Options_create()
    if where == "host":
        a, b = Ah.copy(order="F"), B.copy(order="F")
        pa, pb = a.ctypes.data, b.ctypes.data
    else:
        da, db = to_dev(Ah), to_dev(B)
        pa, pb = da.data_ptr(), db.data_ptr()
    ha = L.slate_HermitianMatrix_create_fromScaLAPACK_r64(uplo, n, pa, n, nb, 1, 1, 0)
    hb = _mat(L, pb, n, nrhs, n, nb)
    L.slate_chol_solve_r64(ha, hb, opts)
    torch.cuda.synchronize()
    assert L.slate_gb300_last_status() == 0 and L.slate_gb300_last_info() == 0
    X = b if where == "host" else to_host(db)
    F = a if where == "host" else to_host(da)
    assert berr(orc, A, X, B, sym=True) <= 3 * EPS
    Lf = np.linalg.cholesky(A)
    ref = Lf if uplo == b"L" else Lf.T
    mask = np.tril(np.ones((n, n), bool)) if uplo == b"L" else np.triu(np.ones((n, n), bool))
    np.testing.assert_allclose(F[mask], ref[mask], atol=1e-12)
    assert (F[~mask] == 7.0).all()                  # the other triangle is untouched
    # solve again with the factor
    b2 = B.copy(order="F")
    hb2 = _mat(L, b2.ctypes.data, n, nrhs, n, nb)
    L.slate_chol_solve_using_factor_r64(ha, hb2, opts)
    assert L.slate_gb300_last_status() == 0
    np.testing.assert_allclose(b2, X, rtol=0, atol=1e-12 * np.abs(X).max())
    for h in (hb, hb2):
        L.slate_Matrix_destroy_r64(h)
    L.slate_HermitianMatrix_destroy_r64(ha)
    L.slate_Options_destroy(opts)


def test_c_api_info(orc, slt):
    L = _api(slt)
    n, nb = 100, 32
    A = orc.generate(2, 75, n, n)
    A[:, 20] = 0.0
    B = orc.generate(2, 76, n, 1)
    opts = L.slate_Options_create()
    ha, hb = _mat(L, A.ctypes.data, n, n, n, nb), _mat(L, B.ctypes.data, n, 1, n, nb)
    L.slate_lu_solve_r64(ha, hb, opts)
    assert L.slate_gb300_last_status() == 0 and L.slate_gb300_last_info() == 21
    S = spd(orc, n, 77)
    S[60, 60] = -1.0
    hs = L.slate_HermitianMatrix_create_fromScaLAPACK_r64(b"L", n, S.ctypes.data, n, nb, 1, 1, 0)
    L.slate_chol_factor_r64(hs, opts)
    assert L.slate_gb300_last_info() == 61
    for h in (ha, hb):
        L.slate_Matrix_destroy_r64(h)
    L.slate_HermitianMatrix_destroy_r64(hs)
    L.slate_Options_destroy(opts)


def _api_more(slt):
    L = _api(slt)
    for name in ("slate_lu_solve_nopiv_r64", "slate_lu_solve_using_factor_nopiv_r64"):
        getattr(L, name).argtypes = [vp, vp, vp]
    L.slate_lu_factor_nopiv_r64.argtypes = [vp, vp]
    L.slate_lu_inverse_using_factor_r64.argtypes = [vp, vp, vp]
    L.slate_lu_inverse_using_factor_out_of_place_r64.argtypes = [vp, vp, vp, vp]
    L.slate_lu_rcondest_using_factor_r64.argtypes = [ctypes.c_char, vp, ctypes.c_double, vp]
    L.slate_lu_rcondest_using_factor_r64.restype = ctypes.c_double
    L.slate_chol_inverse_using_factor_r64.argtypes = [vp, vp]
    L.slate_chol_rcondest_using_factor_r64.argtypes = [ctypes.c_char, vp, ctypes.c_double, vp]
    L.slate_chol_rcondest_using_factor_r64.restype = ctypes.c_double
    L.slate_Options_set_MethodLU.argtypes = [vp, ctypes.c_char]
    return L


def test_c_api_calu_and_nopiv(orc, slt):
    import torch
    L = _api_more(slt)
    n, nb = 256, 64
    A = orc.generate(2, 75, n, n)
    B = orc.generate(2, 76, n, 2)
    # CALU through the option: the same factors as the driver with method_lu "C"
    opts = L.slate_Options_create()
    L.slate_Options_set_MethodLU(opts, b"C")
    a = A.copy(order="F")
    h = _mat(L, a.ctypes.data, n, n, n, nb)
    piv = L.slate_Pivots_create()
    L.slate_lu_factor_r64(h, piv, opts)
    assert L.slate_gb300_last_status() == 0 and L.slate_gb300_last_info() == 0
    dA = to_dev(A)
    slt.getrf(dA, slt.Options(nb=nb, method_lu="C"))
    torch.cuda.synchronize()
    assert np.array_equal(a, to_host(dA))
    # NoPiv forms on a diagonally dominant matrix
    D = np.asfortranarray(A + n * np.eye(n))
    d, b = D.copy(order="F"), B.copy(order="F")
    hd, hb = _mat(L, d.ctypes.data, n, n, n, nb), _mat(L, b.ctypes.data, n, 2, n, nb)
    L.slate_lu_solve_nopiv_r64(hd, hb, None)
    assert L.slate_gb300_last_status() == 0 and L.slate_gb300_last_info() == 0
    assert berr(orc, D, b, B) <= 3 * EPS
    d2, b2 = D.copy(order="F"), B.copy(order="F")
    hd2, hb2 = _mat(L, d2.ctypes.data, n, n, n, nb), _mat(L, b2.ctypes.data, n, 2, n, nb)
    L.slate_lu_factor_nopiv_r64(hd2, None)
    L.slate_lu_solve_using_factor_nopiv_r64(hd2, hb2, None)
    assert L.slate_gb300_last_status() == 0
    assert np.array_equal(b2, b)
    Lf = np.tril(d2, -1) + np.eye(n)
    assert np.abs(Lf @ np.triu(d2) - D).max() <= 1e-12 * np.abs(D).max()
    for x in (h, hd, hb, hd2, hb2):
        L.slate_Matrix_destroy_r64(x)
    L.slate_Pivots_destroy(piv)
    L.slate_Options_destroy(opts)


def test_c_api_inverse_and_rcond(orc, slt):
    import scipy.linalg.lapack as lp
    L = _api_more(slt)
    n, nb = 200, 64
    A = orc.generate(2, 77, n, n)
    a = A.copy(order="F")
    h = _mat(L, a.ctypes.data, n, n, n, nb)
    piv = L.slate_Pivots_create()
    L.slate_lu_factor_r64(h, piv, None)
    anorm = np.abs(A).sum(0).max()
    rc = L.slate_lu_rcondest_using_factor_r64(b"1", h, anorm, None)
    assert L.slate_gb300_last_status() == 0
    lu, _, _ = lp.dgetrf(A)
    ref, _ = lp.dgecon(lu, anorm, norm="1")
    assert abs(rc - ref) <= 0.01 * ref
    ai = np.zeros((n, n), order="F")
    hi = _mat(L, ai.ctypes.data, n, n, n, nb)
    f = a.copy(order="F")
    L.slate_lu_inverse_using_factor_out_of_place_r64(h, piv, hi, None)
    assert L.slate_gb300_last_status() == 0 and np.array_equal(a, f)       # factors kept
    Ainv = np.linalg.inv(A)
    assert np.abs(ai - Ainv).max() <= 1e-10 * np.abs(Ainv).max()
    L.slate_lu_inverse_using_factor_r64(h, piv, None)
    assert np.array_equal(a, ai)
    S = spd(orc, n, 78)
    snorm = np.abs(S).sum(0).max()
    for uplo in (b"L", b"U"):
        s = S.copy(order="F")
        hs = L.slate_HermitianMatrix_create_fromScaLAPACK_r64(uplo, n, s.ctypes.data, n, nb, 1, 1, 0)
        L.slate_chol_factor_r64(hs, None)
        rc = L.slate_chol_rcondest_using_factor_r64(b"1", hs, snorm, None)
        c, _ = lp.dpotrf(S, lower=1)
        ref, _ = lp.dpocon(c, snorm, uplo="L")
        assert abs(rc - ref) <= 0.01 * ref
        L.slate_chol_inverse_using_factor_r64(hs, None)
        assert L.slate_gb300_last_status() == 0 and L.slate_gb300_last_info() == 0
        Si = np.linalg.inv(S)
        tri = np.tril if uplo == b"L" else np.triu
        assert np.abs(tri(s) - tri(Si)).max() <= 1e-10 * np.abs(Si).max()
        L.slate_HermitianMatrix_destroy_r64(hs)
    for x in (h, hi):
        L.slate_Matrix_destroy_r64(x)
    L.slate_Pivots_destroy(piv)
