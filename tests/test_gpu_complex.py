"""Complex (c = complex<float>, z = complex<double>) and the remaining
single-precision forms on the GPU, through the C ABI.

Checks, against LAPACK (scipy) and numpy on the host:
* getrf: pivots identical to LAPACK's xgetrf wherever the pivot margin
  (largest / second-largest cabs1 = |re| + |im| of the eliminated column)
  exceeds rounding, factors close; info at an exactly zero column;
* gesv: SLATE's tester residual ||B - A X||_1 / (n ||A||_1 ||X||_1) <= 3 eps
  (z) and <= 50 eps (c, the tester's tolerance, test/test.cc:356);
* getrs with trans 'N', 'T', 'C'; potrf against numpy's Cholesky, posv, info
  of a non-positive-definite matrix; zcgesv iteration counts and fallback;
* the LAPACK-compatible host entry points and the C API handles of these
  precisions.
"""
import ctypes

import numpy as np
import pytest

from gpu_util import to_dev, to_host

pytestmark = pytest.mark.gpu

EPS = {np.complex64: np.finfo(np.float32).eps, np.complex128: np.finfo(np.float64).eps,
       np.float32: np.finfo(np.float32).eps, np.float64: np.finfo(np.float64).eps}


def _rand(orc, n, m, seed, dt):
    re = orc.generate(2, seed, n, m)
    if np.issubdtype(dt, np.complexfloating):
        im = orc.generate(2, seed + 1000, n, m)
        return np.asfortranarray((re + 1j * im).astype(dt))
    return np.asfortranarray(re.astype(dt))


def _hpd(orc, n, seed, dt):
    G = _rand(orc, n, n, seed, np.complex128 if np.issubdtype(dt, np.complexfloating) else np.float64)
    A = G @ G.conj().T / n + np.eye(n)
    return np.asfortranarray(A.astype(dt))


def _berr(A, X, B):
    A, X, B = (np.asarray(v, dtype=np.complex128) for v in (A, X, B))
    n = A.shape[0]
    R = B - A @ X
    return np.abs(R).sum(0).max() / (n * np.abs(A).sum(0).max() * np.abs(X).sum(0).max())


def _lu_margins(A):
    """Partial-pivoting LU in complex128 with cabs1: per column the ratio of the
    largest to the second-largest candidate (inf when alone)."""
    A = np.array(A, dtype=np.complex128)
    m, n = A.shape
    mg = np.full(min(m, n), np.inf)
    for j in range(min(m, n)):
        c = np.abs(A[j:, j].real) + np.abs(A[j:, j].imag)
        p = int(np.argmax(c))
        if len(c) > 1:
            s = np.sort(c)[::-1]
            mg[j] = s[0] / s[1] if s[1] > 0 else np.inf
        if p:
            A[[j, j + p]] = A[[j + p, j]]
        if A[j, j] != 0:
            A[j + 1:, j] /= A[j, j]
            A[j + 1:, j + 1:] -= np.outer(A[j + 1:, j], A[j, j + 1:])
    return mg


@pytest.mark.parametrize("dt", [np.complex64, np.complex128])
@pytest.mark.parametrize("m,n,nb", [(1, 1, 16), (7, 7, 4), (100, 100, 32), (300, 300, 64), (517, 400, 128),
                                    (400, 517, 128), (1000, 1000, 256)])
def test_complex_getrf_matches_lapack(orc, slt, dt, m, n, nb):
    import scipy.linalg.lapack as la
    import torch
    A = _rand(orc, m, n, 11 + m, dt)
    dA = to_dev(A)
    info, ipiv = slt.getrf(dA, slt.Options(nb=nb))
    torch.cuda.synchronize()
    f = la.cgetrf if dt == np.complex64 else la.zgetrf
    lu, lip, linfo = f(A.copy())
    assert info == linfo == 0
    gip = np.asarray(slt.ipiv_to_lapack(ipiv, nb)).astype(np.int64)
    robust = _lu_margins(A) > 1 + 1e3 * max(m, n) * EPS[dt]
    assert np.array_equal(gip[robust], (lip + 1)[robust])
    if np.array_equal(gip, lip + 1):
        tol = 5e-3 if dt == np.complex64 else 1e-10
        assert np.abs(to_host(dA) - lu).max() <= tol * max(1.0, np.abs(lu).max())


@pytest.mark.parametrize("dt", [np.complex64, np.complex128])
def test_complex_getrf_zero_column_info(orc, slt, dt):
    import torch
    n = 80
    A = _rand(orc, n, n, 5, dt)
    A[:, 17] = 0
    dA = to_dev(A)
    info, _ = slt.getrf(dA, slt.Options(nb=32))
    torch.cuda.synchronize()
    assert info == 18


@pytest.mark.parametrize("dt", [np.complex64, np.complex128])
@pytest.mark.parametrize("n,nb,nrhs", [(33, 16, 1), (500, 128, 3), (1100, 256, 5)])
def test_complex_gesv_backward_error(orc, slt, dt, n, nb, nrhs):
    import torch
    A = _rand(orc, n, n, 21 + n, dt)
    B = _rand(orc, n, nrhs, 22 + n, dt)
    dA, dB = to_dev(A), to_dev(B)
    info, _ = slt.gesv(dA, dB, slt.Options(nb=nb))
    torch.cuda.synchronize()
    assert info == 0
    bound = (3 if dt == np.complex128 else 50) * EPS[dt]
    assert _berr(A, to_host(dB), B) <= bound


@pytest.mark.parametrize("dt", [np.complex64, np.complex128, np.float32])
@pytest.mark.parametrize("trans", ["N", "T", "C"])
def test_getrs_trans_against_numpy(orc, slt, dt, trans):
    import torch
    n, nb, nrhs = 300, 64, 4
    A = _rand(orc, n, n, 31, dt)
    B = _rand(orc, n, nrhs, 32, dt)
    dA = to_dev(A)
    info, ipiv = slt.getrf(dA, slt.Options(nb=nb))
    dB = to_dev(B)
    slt.getrs(dA, ipiv, dB, slt.Options(nb=nb), trans=trans)
    torch.cuda.synchronize()
    X = to_host(dB)
    op = A if trans == "N" else (A.T if trans == "T" else A.conj().T)
    assert _berr(op, X, B) <= 50 * EPS[dt]


@pytest.mark.parametrize("dt", [np.complex64, np.complex128, np.float32])
@pytest.mark.parametrize("n,nb", [(1, 16), (70, 16), (300, 64), (777, 256)])
def test_potrf_and_posv(orc, slt, dt, n, nb):
    import torch
    A = _hpd(orc, n, 41 + n, dt)
    dA = to_dev(A)
    info = slt.potrf(dA, slt.Options(nb=nb))
    torch.cuda.synchronize()
    assert info == 0
    L = np.tril(to_host(dA))
    Lr = np.linalg.cholesky(A.astype(np.complex128 if np.issubdtype(dt, np.complexfloating) else np.float64))
    tol = 1e-3 if dt in (np.complex64, np.float32) else 1e-11
    assert np.abs(L - Lr).max() <= tol
    B = _rand(orc, n, 3, 42 + n, dt)
    dA2, dB = to_dev(A), to_dev(B)
    assert slt.posv(dA2, dB, slt.Options(nb=nb)) == 0
    torch.cuda.synchronize()
    assert _berr(A, to_host(dB), B) <= (3 if dt == np.complex128 else 50) * EPS[dt]


@pytest.mark.parametrize("dt", [np.complex64, np.complex128])
def test_potrf_not_positive_definite(orc, slt, dt):
    import torch
    n = 90
    A = _hpd(orc, n, 7, dt)
    A[40, 40] = -5.0
    dA = to_dev(A)
    info = slt.potrf(dA, slt.Options(nb=32))
    torch.cuda.synchronize()
    # the leading 40 x 40 block is HPD; the minor of order 41 is not
    assert info == 41


def test_zcgesv_converges_and_falls_back(orc, slt):
    import torch
    n, nb, nrhs = 600, 128, 2
    A = _rand(orc, n, n, 51, np.complex128)
    B = _rand(orc, n, nrhs, 52, np.complex128)
    dA, dB = to_dev(A), to_dev(B)
    dX = to_dev(np.zeros((n, nrhs), dtype=np.complex128))
    info, it, _ = slt.gesv_mixed(dA, dB, dX, slt.Options(nb=nb))
    torch.cuda.synchronize()
    assert info == 0 and it >= 0
    assert _berr(A, to_host(dX), B) <= 3 * n * EPS[np.complex128]
    assert np.array_equal(to_host(dA), A)                 # converged: A untouched
    # no refinement allowed: SLATE's fallback code -(itermax + 1) = -1, FP64 LU
    dA, dX = to_dev(A), to_dev(np.zeros((n, nrhs), dtype=np.complex128))
    info, it, _ = slt.gesv_mixed(dA, dB, dX, slt.Options(nb=nb, max_iterations=0))
    torch.cuda.synchronize()
    assert info == 0 and it == -1
    assert _berr(A, to_host(dX), B) <= 3 * EPS[np.complex128]


# ---------------------------------------------------------------------------
# host entry points (LAPACK-compatible and C API)
def _c(x):
    return ctypes.byref(ctypes.c_int(x))


@pytest.mark.parametrize("p,dt", [("c", np.complex64), ("z", np.complex128)])
def test_lapack_complex_gesv_getrf_getrs(orc, slt, p, dt):
    L = slt.lib()
    n, nrhs = 257, 2
    A = _rand(orc, n, n, 61, dt)
    B = _rand(orc, n, nrhs, 62, dt)
    a, b = A.copy(order="F"), B.copy(order="F")
    ipiv = np.zeros(n, np.int32)
    info = ctypes.c_int(-9)
    getattr(L, "slate_%sgesv" % p)(_c(n), _c(nrhs), a.ctypes.data_as(ctypes.c_void_p), _c(n),
                                    ipiv.ctypes.data_as(ctypes.c_void_p), b.ctypes.data_as(ctypes.c_void_p), _c(n),
                                    ctypes.byref(info))
    assert info.value == 0
    assert _berr(A, b, B) <= (3 if p == "z" else 50) * EPS[dt]
    # getrf + getrs('C') through the underscore manglings
    a2 = A.copy(order="F")
    ip2 = np.zeros(n, np.int32)
    getattr(L, "slate_%sgetrf_" % p)(_c(n), _c(n), a2.ctypes.data_as(ctypes.c_void_p), _c(n),
                                      ip2.ctypes.data_as(ctypes.c_void_p), ctypes.byref(info))
    assert info.value == 0 and np.array_equal(ip2, ipiv)
    b2 = B.copy(order="F")
    getattr(L, "slate_%sgetrs_" % p)(ctypes.c_char_p(b"C"), _c(n), _c(nrhs), a2.ctypes.data_as(ctypes.c_void_p),
                                      _c(n), ip2.ctypes.data_as(ctypes.c_void_p), b2.ctypes.data_as(ctypes.c_void_p),
                                      _c(n), ctypes.byref(info))
    assert info.value == 0
    assert _berr(A.conj().T, b2, B) <= (3 if p == "z" else 50) * EPS[dt]


@pytest.mark.parametrize("p,dt", [("s", np.float32), ("c", np.complex64), ("z", np.complex128)])
@pytest.mark.parametrize("uplo", [b"L", b"U"])
def test_lapack_posv_potrf(orc, slt, p, dt, uplo):
    L = slt.lib()
    n, nrhs = 200, 3
    A = _hpd(orc, n, 71, dt)
    B = _rand(orc, n, nrhs, 72, dt)
    keep = np.tril(np.ones((n, n), bool)) if uplo == b"L" else np.triu(np.ones((n, n), bool))
    a = np.asfortranarray(np.where(keep, A, 7.0).astype(dt))     # the other triangle holds a marker
    b = B.copy(order="F")
    info = ctypes.c_int(-9)
    getattr(L, "slate_%sposv" % p)(ctypes.c_char_p(uplo), _c(n), _c(nrhs), a.ctypes.data_as(ctypes.c_void_p), _c(n),
                                    b.ctypes.data_as(ctypes.c_void_p), _c(n), ctypes.byref(info))
    assert info.value == 0
    assert _berr(A, b, B) <= (3 if p == "z" else 50) * EPS[dt]
    assert np.all(a[~keep] == 7.0)                                   # only the referenced triangle written
    F = np.where(keep, a, 0)
    LL = F @ F.conj().T if uplo == b"L" else F.conj().T @ F
    assert np.abs(LL - A).max() <= (1e-3 if p in "sc" else 1e-11) * np.abs(A).max()
    a3 = np.asfortranarray(np.where(keep, A, 7.0).astype(dt))
    getattr(L, "slate_%spotrf_" % p)(ctypes.c_char_p(uplo), _c(n), a3.ctypes.data_as(ctypes.c_void_p), _c(n),
                                      ctypes.byref(info))
    assert info.value == 0 and np.allclose(a3, a)


def test_lapack_zcgesv_and_sgetrs(orc, slt):
    L = slt.lib()
    n, nrhs = 300, 2
    A = _rand(orc, n, n, 81, np.complex128)
    B = _rand(orc, n, nrhs, 82, np.complex128)
    a, b = A.copy(order="F"), B.copy(order="F")
    x = np.zeros((n, nrhs), dtype=np.complex128, order="F")
    ipiv = np.zeros(n, np.int32)
    it, info = ctypes.c_int(-99), ctypes.c_int(-9)
    L.slate_zcgesv(_c(n), _c(nrhs), a.ctypes.data_as(ctypes.c_void_p), _c(n), ipiv.ctypes.data_as(ctypes.c_void_p),
                   b.ctypes.data_as(ctypes.c_void_p), _c(n), x.ctypes.data_as(ctypes.c_void_p), _c(n), None, None,
                   ctypes.byref(it), ctypes.byref(info))
    assert info.value == 0 and it.value >= 0
    assert _berr(A, x, B) <= 3 * n * EPS[np.complex128]
    # sgetrs 'T' on sgetrf's factors
    As = _rand(orc, n, n, 83, np.float32)
    Bs = _rand(orc, n, nrhs, 84, np.float32)
    a = As.copy(order="F")
    ip = np.zeros(n, np.int32)
    L.slate_sgetrf(_c(n), _c(n), a.ctypes.data_as(ctypes.c_void_p), _c(n), ip.ctypes.data_as(ctypes.c_void_p),
                   ctypes.byref(info))
    assert info.value == 0
    b = Bs.copy(order="F")
    L.slate_sgetrs(ctypes.c_char_p(b"T"), _c(n), _c(nrhs), a.ctypes.data_as(ctypes.c_void_p), _c(n),
                   ip.ctypes.data_as(ctypes.c_void_p), b.ctypes.data_as(ctypes.c_void_p), _c(n), ctypes.byref(info))
    assert info.value == 0
    assert _berr(As.T, b, Bs) <= 50 * EPS[np.float32]


@pytest.mark.parametrize("R,dt", [("c64", np.complex128), ("c32", np.complex64)])
def test_c_api_complex_lu_and_chol(orc, slt, R, dt):
    L = slt.lib()
    i64, vp = ctypes.c_int64, ctypes.c_void_p
    for f in ("slate_Matrix_create_fromScaLAPACK_", "slate_HermitianMatrix_create_fromScaLAPACK_"):
        getattr(L, f + R).restype = vp
    L.slate_Matrix_create_fromScaLAPACK_c64.argtypes = [i64, i64, vp, i64, i64, i64, ctypes.c_int, ctypes.c_int, vp]
    L.slate_Matrix_create_fromScaLAPACK_c32.argtypes = [i64, i64, vp, i64, i64, i64, ctypes.c_int, ctypes.c_int, vp]
    L.slate_HermitianMatrix_create_fromScaLAPACK_c64.argtypes = [ctypes.c_char, i64, vp, i64, i64, ctypes.c_int,
                                                                  ctypes.c_int, vp]
    L.slate_HermitianMatrix_create_fromScaLAPACK_c32.argtypes = [ctypes.c_char, i64, vp, i64, i64, ctypes.c_int,
                                                                  ctypes.c_int, vp]
    L.slate_gb300_last_info.restype = i64
    n, nrhs, nb = 260, 2, 64
    tol = (3 if dt == np.complex128 else 50) * EPS[dt]
    A = _rand(orc, n, n, 91, dt)
    B = _rand(orc, n, nrhs, 92, dt)
    a, b = A.copy(order="F"), B.copy(order="F")
    opts = vp(L.slate_Options_create())
    ha = vp(getattr(L, "slate_Matrix_create_fromScaLAPACK_" + R)(n, n, a.ctypes.data, n, nb, nb, 1, 1, None))
    hb = vp(getattr(L, "slate_Matrix_create_fromScaLAPACK_" + R)(n, nrhs, b.ctypes.data, n, nb, nb, 1, 1, None))
    getattr(L, "slate_lu_solve_" + R)(ha, hb, opts)
    assert L.slate_gb300_last_status() == 0 and L.slate_gb300_last_info() == 0
    assert _berr(A, b, B) <= tol
    getattr(L, "slate_Matrix_destroy_" + R)(ha)
    getattr(L, "slate_Matrix_destroy_" + R)(hb)
    for uplo in (b"L", b"U"):
        H = _hpd(orc, n, 93, dt)
        keep = np.tril(np.ones((n, n), bool)) if uplo == b"L" else np.triu(np.ones((n, n), bool))
        h = np.asfortranarray(np.where(keep, H, 7.0).astype(dt))
        b = B.copy(order="F")
        hh = vp(getattr(L, "slate_HermitianMatrix_create_fromScaLAPACK_" + R)(uplo, n, h.ctypes.data, n, nb, 1, 1,
                                                                              None))
        hb = vp(getattr(L, "slate_Matrix_create_fromScaLAPACK_" + R)(n, nrhs, b.ctypes.data, n, nb, nb, 1, 1, None))
        getattr(L, "slate_chol_solve_" + R)(hh, hb, opts)
        assert L.slate_gb300_last_status() == 0 and L.slate_gb300_last_info() == 0
        assert _berr(H, b, B) <= tol
        assert np.all(h[~keep] == 7.0)
        getattr(L, "slate_HermitianMatrix_destroy_" + R)(hh)
        getattr(L, "slate_Matrix_destroy_" + R)(hb)
    L.slate_Options_destroy(opts)


def test_c_api_chol_r32(orc, slt):
    L = slt.lib()
    i64, vp = ctypes.c_int64, ctypes.c_void_p
    L.slate_HermitianMatrix_create_fromScaLAPACK_r32.restype = vp
    L.slate_HermitianMatrix_create_fromScaLAPACK_r32.argtypes = [ctypes.c_char, i64, vp, i64, i64, ctypes.c_int,
                                                                  ctypes.c_int, vp]
    L.slate_Matrix_create_fromScaLAPACK_r32.restype = vp
    L.slate_Matrix_create_fromScaLAPACK_r32.argtypes = [i64, i64, vp, i64, i64, i64, ctypes.c_int, ctypes.c_int, vp]
    L.slate_gb300_last_info.restype = i64
    n, nrhs, nb = 300, 3, 64
    A = _hpd(orc, n, 95, np.float32)
    B = _rand(orc, n, nrhs, 96, np.float32)
    a, b = A.copy(order="F"), B.copy(order="F")
    opts = vp(L.slate_Options_create())
    ha = vp(L.slate_HermitianMatrix_create_fromScaLAPACK_r32(b"L", n, a.ctypes.data, n, nb, 1, 1, None))
    hb = vp(L.slate_Matrix_create_fromScaLAPACK_r32(n, nrhs, b.ctypes.data, n, nb, nb, 1, 1, None))
    L.slate_chol_factor_r32(ha, opts)
    assert L.slate_gb300_last_status() == 0 and L.slate_gb300_last_info() == 0
    L.slate_chol_solve_using_factor_r32(ha, hb, opts)
    assert L.slate_gb300_last_status() == 0
    assert _berr(A, b, B) <= 50 * EPS[np.float32]
    L.slate_HermitianMatrix_destroy_r32(ha)
    L.slate_Matrix_destroy_r32(hb)
    L.slate_Options_destroy(opts)
