"""ctypes wrapper over the CPU oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY: the test suite, the package smoke check and the
benchmark's CPU-baseline leg use this module as the checker.  Product code
never imports it.

Every function restates the SLATE routine cited in oracle/oracle.cc.
Matrices are numpy arrays in Fortran (column-major) order.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_REF = None

i64 = ctypes.c_int64
dbl = ctypes.c_double
vp = ctypes.c_void_p


def build():
    subprocess.check_call(["bash", os.path.join(_HERE, "build.sh")],
                          stdout=subprocess.DEVNULL)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        L.orc_dgetrf.restype = i64
        L.orc_sgetrf.restype = i64
        L.orc_dgesv.restype = i64
        L.orc_dpotrf.restype = i64
        L.orc_spotrf.restype = i64
        L.orc_dposv.restype = i64
        L.orc_dgesv_mixed.restype = i64
        L.orc_dposv_mixed.restype = i64
        L.orc_dgesv_mixed_gmres.restype = i64
        L.orc_dposv_mixed_gmres.restype = i64
        L.orc_backward_error.restype = dbl
        L.orc_get_threads.restype = ctypes.c_int
        _LIB = L
    return _LIB


def ref_lib():
    """SLATE's own matgen/random.cc built by oracle/build_ref.sh, or None."""
    global _REF
    if _REF is None:
        path = os.path.join(_HERE, "_ref", "libref_random.so")
        if not os.path.exists(path):
            return None
        _REF = ctypes.CDLL(path)
    return _REF


def _p(a):
    return a.ctypes.data_as(vp)


def set_threads(n):
    lib().orc_set_threads(ctypes.c_int(int(n)))


def get_threads():
    return int(lib().orc_get_threads())


def use_host_blas():
    """Route the oracle's tile gemm through scipy's bundled BLAS if present."""
    try:
        import scipy.linalg.cython_blas as cb
    except Exception:
        return False
    get = ctypes.pythonapi.PyCapsule_GetPointer
    get.restype = ctypes.c_void_p
    get.argtypes = [ctypes.py_object, ctypes.c_char_p]
    capi = cb.__pyx_capi__
    try:
        import scipy.linalg.cython_lapack as cl
        pd = get(capi["dgemm"], _capsule_name(capi["dgemm"]))
        ps = get(capi["sgemm"], _capsule_name(capi["sgemm"]))
        td = get(capi["dtrsm"], _capsule_name(capi["dtrsm"]))
        ts = get(capi["strsm"], _capsule_name(capi["strsm"]))
        lcapi = cl.__pyx_capi__
        fd = get(lcapi["dpotrf"], _capsule_name(lcapi["dpotrf"]))
        fs = get(lcapi["spotrf"], _capsule_name(lcapi["spotrf"]))
    except Exception:
        return False
    lib().orc_set_blas(ctypes.c_void_p(pd), ctypes.c_void_p(ps))
    lib().orc_set_lapack(ctypes.c_void_p(td), ctypes.c_void_p(ts), ctypes.c_void_p(fd), ctypes.c_void_p(fs))
    return True


def _capsule_name(cap):
    f = ctypes.pythonapi.PyCapsule_GetName
    f.restype = ctypes.c_char_p
    f.argtypes = [ctypes.py_object]
    return f(cap)


def use_builtin_blas():
    lib().orc_set_blas(None, None)
    lib().orc_set_lapack(None, None, None, None)


def philox(s0, s1, key):
    out = (ctypes.c_uint64 * 2)()
    lib().orc_philox(ctypes.c_uint64(s0), ctypes.c_uint64(s1), ctypes.c_uint64(key), out)
    return int(out[0]), int(out[1])


def generate(dist, seed, m, n, ioff=0, joff=0, dtype=np.float64):
    """slate::random::generate (matgen/random.cc:197-230).  dist codes:
    1 uniform, 2 uniform signed, 3 normal, 4 unit disk, 5 unit circle,
    6 binary, 7 binary signed."""
    A = np.zeros((m, n), dtype=dtype, order="F")
    f = lib().orc_generate_d if dtype == np.float64 else lib().orc_generate_s
    f(ctypes.c_int(dist), i64(seed), i64(m), i64(n), i64(ioff), i64(joff), _p(A), i64(max(m, 1)))
    return A


def ref_generate(dist, seed, m, n, ioff=0, joff=0, dtype=np.float64):
    R = ref_lib()
    if R is None:
        return None
    A = np.zeros((m, n), dtype=dtype, order="F")
    f = R.ref_generate_d if dtype == np.float64 else R.ref_generate_s
    f(ctypes.c_int(dist), i64(seed), i64(m), i64(n), i64(ioff), i64(joff), _p(A), i64(max(m, 1)))
    return A


KINDS = {"zeros": 0, "ones": 1, "identity": 2, "ij": 3, "jordan": 4, "jordanT": 5,
         "kms": 6, "minij": 7, "hilb": 8, "lehmer": 9, "lotkin": 10}


def generate_kind(kind, m, n):
    A = np.zeros((m, n), order="F")
    rc = lib().orc_generate_kind(ctypes.c_int(KINDS[kind]), i64(m), i64(n), _p(A), i64(max(m, 1)))
    assert rc == 0
    return A


def getrf(A, nb, ib=16, panel_threads=1, threshold=1.0, margins=False):
    """LU with partial pivoting in place.  Returns (info, piv_tile, piv_off,
    ipiv (1-based), margin or None)."""
    assert A.flags.f_contiguous
    m, n = A.shape
    mn = min(m, n)
    pt = np.zeros(max(mn, 1), np.int64)
    po = np.zeros(max(mn, 1), np.int64)
    ip = np.zeros(max(mn, 1), np.int64)
    mg = np.zeros(max(mn, 1), np.float64) if margins else None
    f = lib().orc_dgetrf if A.dtype == np.float64 else lib().orc_sgetrf
    info = f(i64(m), i64(n), _p(A), i64(max(m, 1)), i64(nb), i64(ib), ctypes.c_int(panel_threads),
             dbl(threshold), _p(pt), _p(po), _p(ip), _p(mg) if margins else None)
    return int(info), pt[:mn], po[:mn], ip[:mn], (mg[:mn] if margins else None)


def getrs(LU, piv_tile, piv_off, B, nb):
    n = LU.shape[0]
    nrhs = B.shape[1]
    lib().orc_dgetrs(i64(n), i64(nrhs), _p(LU), i64(n), _p(np.ascontiguousarray(piv_tile)),
                     _p(np.ascontiguousarray(piv_off)), i64(nb), _p(B), i64(n))


def gesv(A, B, nb, ib=16, panel_threads=1):
    n = A.shape[0]
    pt = np.zeros(n, np.int64)
    po = np.zeros(n, np.int64)
    info = lib().orc_dgesv(i64(n), i64(B.shape[1]), _p(A), i64(n), i64(nb), i64(ib),
                           ctypes.c_int(panel_threads), _p(pt), _p(po), _p(B), i64(n))
    return int(info), pt, po


def potrf(A, nb):
    f = lib().orc_dpotrf if A.dtype == np.float64 else lib().orc_spotrf
    return int(f(i64(A.shape[0]), _p(A), i64(A.shape[0]), i64(nb)))


def potrs(L, B, nb):
    n = L.shape[0]
    lib().orc_dpotrs(i64(n), i64(B.shape[1]), _p(L), i64(n), i64(nb), _p(B), i64(n))


def posv(A, B, nb):
    n = A.shape[0]
    return int(lib().orc_dposv(i64(n), i64(B.shape[1]), _p(A), i64(n), i64(nb), _p(B), i64(n)))


def gesv_mixed(A, B, nb, ib=16, itermax=30, tol=0.0, use_fallback=True, panel_threads=1):
    n, nrhs = B.shape
    X = np.zeros((n, nrhs), order="F")
    pt = np.zeros(n, np.int64)
    po = np.zeros(n, np.int64)
    it = i64(0)
    info = lib().orc_dgesv_mixed(i64(n), i64(nrhs), _p(A), i64(n), _p(pt), _p(po), _p(B), i64(n),
                                 _p(X), i64(n), i64(nb), i64(ib), ctypes.c_int(panel_threads),
                                 i64(itermax), dbl(tol), ctypes.c_int(int(use_fallback)),
                                 ctypes.byref(it))
    return int(info), X, int(it.value), pt, po


def posv_mixed(A, B, nb, itermax=30, tol=0.0, use_fallback=True):
    n, nrhs = B.shape
    X = np.zeros((n, nrhs), order="F")
    it = i64(0)
    info = lib().orc_dposv_mixed(i64(n), i64(nrhs), _p(A), i64(n), _p(B), i64(n), _p(X), i64(n),
                                 i64(nb), i64(itermax), dbl(tol), ctypes.c_int(int(use_fallback)),
                                 ctypes.byref(it))
    return int(info), X, int(it.value)


def gesv_mixed_gmres(A, b, nb, ib=16, itermax=30, tol=0.0, use_fallback=True, panel_threads=1):
    n = A.shape[0]
    b = np.asfortranarray(b.reshape(n, 1))
    X = np.zeros((n, 1), order="F")
    pt = np.zeros(n, np.int64)
    po = np.zeros(n, np.int64)
    it = i64(0)
    info = lib().orc_dgesv_mixed_gmres(i64(n), _p(A), i64(n), _p(pt), _p(po), _p(b), _p(X),
                                       i64(nb), i64(ib), ctypes.c_int(panel_threads),
                                       i64(itermax), dbl(tol), ctypes.c_int(int(use_fallback)),
                                       ctypes.byref(it))
    return int(info), X, int(it.value)


def posv_mixed_gmres(A, b, nb, itermax=30, tol=0.0, use_fallback=True):
    n = A.shape[0]
    b = np.asfortranarray(b.reshape(n, 1))
    X = np.zeros((n, 1), order="F")
    it = i64(0)
    info = lib().orc_dposv_mixed_gmres(i64(n), _p(A), i64(n), _p(b), _p(X), i64(nb),
                                       i64(itermax), dbl(tol), ctypes.c_int(int(use_fallback)),
                                       ctypes.byref(it))
    return int(info), X, int(it.value)


def backward_error(A, X, B, sym_lower=False):
    """||B - A X||_1 / (n ||A||_1 ||X||_1), the SLATE tester's check."""
    n, nrhs = X.shape
    A = np.asfortranarray(A)
    X = np.asfortranarray(X)
    B = np.asfortranarray(B)
    return float(lib().orc_backward_error(i64(n), i64(nrhs), _p(A), i64(A.shape[0]),
                                          ctypes.c_int(int(sym_lower)), _p(X), i64(n), _p(B),
                                          i64(n)))
