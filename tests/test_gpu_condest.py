"""Transposed getrs and the condition estimators (gecondest / pocondest) on
the GPU, against LAPACK (scipy's dgecon / dpocon: the same Hager-Higham
estimator on the same kind of factors) and the exact condition number.

Bar: A^T X = B to backward error <= 3 eps64; rcond within 1 % of LAPACK's
estimate and never below the true 1 / kappa (an estimate of ||A^{-1}|| is a
lower bound).
"""
import numpy as np
import pytest

from gpu_util import EPS, spd, to_dev, to_host

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,nb", [(1, 8), (37, 16), (700, 128)])
def test_getrs_trans(orc, slt, n, nb):
    import torch
    A = orc.generate(2, 91, n, n)
    B = orc.generate(2, 92, n, 3)
    dA, dB = to_dev(A), to_dev(B)
    info, ipiv = slt.getrf(dA, slt.Options(nb=nb))
    slt.getrs(dA, ipiv, dB, slt.Options(nb=nb), trans="T")
    torch.cuda.synchronize()
    assert info == 0
    X = to_host(dB)
    r = B - A.T @ X
    assert np.abs(r).sum(0).max() / (n * np.abs(A.T).sum(0).max() * np.abs(X).sum(0).max()) <= 3 * EPS


@pytest.mark.parametrize("norm", ["1", "I"])
@pytest.mark.parametrize("n", [5, 300])
def test_gecondest_matches_lapack(orc, slt, n, norm):
    import scipy.linalg.lapack as lp
    import torch
    A = orc.generate(2, 93, n, n)
    anorm = np.abs(A).sum(0).max() if norm == "1" else np.abs(A).sum(1).max()
    dA = to_dev(A)
    info, ipiv = slt.getrf(dA, slt.Options(nb=64))
    rc = slt.gecondest(dA, ipiv, anorm, norm, slt.Options(nb=64))
    torch.cuda.synchronize()
    lu, piv, linfo = lp.dgetrf(A)
    rc_lapack, _ = lp.dgecon(lu, anorm, norm=norm)
    kappa = np.linalg.cond(A, 1 if norm == "1" else np.inf)
    assert abs(rc - rc_lapack) <= 0.01 * rc_lapack
    assert rc >= (1 - 1e-8) / kappa


def test_pocondest_matches_lapack(orc, slt):
    import scipy.linalg.lapack as lp
    import torch
    n = 400
    A = spd(orc, n, 94)
    anorm = np.abs(A).sum(0).max()
    dA = to_dev(A)
    assert slt.potrf(dA, slt.Options(nb=64)) == 0
    rc = slt.pocondest(dA, anorm, "1", slt.Options(nb=64))
    torch.cuda.synchronize()
    c, cinfo = lp.dpotrf(A, lower=1)
    rc_lapack, _ = lp.dpocon(c, anorm, uplo="L")
    assert abs(rc - rc_lapack) <= 0.01 * rc_lapack
    assert rc >= (1 - 1e-8) / np.linalg.cond(A, 1)


def test_getri_potri(orc, slt):
    import torch
    n = 260
    A = orc.generate(2, 95, n, n)
    dA = to_dev(A)
    info, ipiv = slt.getrf(dA, slt.Options(nb=64))
    L = slt.lib()
    import ctypes
    f = L.slt_dgetri_device
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.POINTER(ctypes.c_int64)]
    po, _ = slt._opts(slt.Options(nb=64))
    inf = ctypes.c_int64(0)
    assert f(n, dA.data_ptr(), n, ipiv.data_ptr(), po, slt._stream(), ctypes.byref(inf)) == 0
    torch.cuda.synchronize()
    Ainv = to_host(dA)
    assert inf.value == 0
    assert np.abs(Ainv @ A - np.eye(n)).max() <= 1e-10 * np.linalg.cond(A, 1)
    S = spd(orc, n, 96)
    dS = to_dev(S)
    assert slt.potrf(dS, slt.Options(nb=64)) == 0
    g = L.slt_dpotri_device
    g.restype = ctypes.c_int
    g.argtypes = [ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.POINTER(ctypes.c_int64)]
    assert g(n, dS.data_ptr(), n, po, slt._stream(), ctypes.byref(inf)) == 0
    torch.cuda.synchronize()
    Sl = np.tril(to_host(dS))
    Sinv = Sl + np.tril(Sl, -1).T
    assert np.abs(Sinv @ S - np.eye(n)).max() <= 1e-11


def test_lapack_getri_potri_gecon_pocon(orc, slt):
    import ctypes
    import scipy.linalg.lapack as lp
    L = slt.lib()
    c = ctypes.c_int
    n = 150
    A = orc.generate(2, 97, n, n)
    lu, piv, _ = lp.dgetrf(A)
    a = np.asfortranarray(lu.copy())
    ip = (piv + 1).astype(np.int32)
    info = c(0)
    L.slate_dgetri(ctypes.byref(c(n)), a.ctypes.data_as(ctypes.c_void_p), ctypes.byref(c(n)),
                   ip.ctypes.data_as(ctypes.c_void_p), None, None, ctypes.byref(info))
    assert info.value == 0
    assert np.abs(a @ A - np.eye(n)).max() <= 1e-10 * np.linalg.cond(A, 1)
    anorm = np.abs(A).sum(0).max()
    rc = ctypes.c_double(0)
    lu2 = np.asfortranarray(lu.copy())
    L.slate_dgecon(ctypes.c_char_p(b"1"), ctypes.byref(c(n)), lu2.ctypes.data_as(ctypes.c_void_p),
                   ctypes.byref(c(n)), ctypes.byref(ctypes.c_double(anorm)), ctypes.byref(rc), None, None,
                   ctypes.byref(info))
    ref, _ = lp.dgecon(lu, anorm, norm="1")
    assert info.value == 0 and abs(rc.value - ref) <= 0.01 * ref
    S = spd(orc, n, 98)
    ch, _ = lp.dpotrf(S, lower=0)
    for uplo, fac in ((b"U", ch), (b"L", np.asfortranarray(ch.T))):
        s = np.asfortranarray(np.where(np.triu(np.ones((n, n))) if uplo == b"U" else np.tril(np.ones((n, n))), fac, 0.0))
        L.slate_dpotri(ctypes.c_char_p(uplo), ctypes.byref(c(n)), s.ctypes.data_as(ctypes.c_void_p),
                       ctypes.byref(c(n)), ctypes.byref(info))
        assert info.value == 0
        T = np.triu(s) if uplo == b"U" else np.tril(s)
        Sinv = T + (np.triu(T, 1).T if uplo == b"U" else np.tril(T, -1).T)
        assert np.abs(Sinv @ S - np.eye(n)).max() <= 1e-11
    sn = np.abs(S).sum(0).max()
    L.slate_dpocon(ctypes.c_char_p(b"U"), ctypes.byref(c(n)), np.asfortranarray(ch).ctypes.data_as(ctypes.c_void_p),
                   ctypes.byref(c(n)), ctypes.byref(ctypes.c_double(sn)), ctypes.byref(rc), None, None,
                   ctypes.byref(info))
    ref, _ = lp.dpocon(ch, sn, uplo="U")
    assert info.value == 0 and abs(rc.value - ref) <= 0.01 * ref
