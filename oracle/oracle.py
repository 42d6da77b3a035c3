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
        L.orc_dposv_mixed_gmres_nrhs.restype = i64
        L.orc_dgesv_mixed_gmres_nrhs.restype = i64
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


_REF_GETRF = None


def ref_getrf_lib():
    """SLATE's own tile LU panel (src/internal/Tile_getrf.hh) built by
    oracle/build_ref.sh, or None."""
    global _REF_GETRF
    if _REF_GETRF is None:
        path = os.path.join(_HERE, "_ref", "libref_getrf.so")
        if not os.path.exists(path):
            return None
        L = ctypes.CDLL(path)
        for f in (L.ref_getrf_panel_d, L.ref_getrf_d):
            f.restype = i64
        _REF_GETRF = L
    return _REF_GETRF


def ref_getrf_panel(A, nb, ib, threshold=1.0, threads=1):
    """SLATE's tile::getrf on the m x nb panel A (tiles of nb rows), run by
    `threads` panel threads as internal::getrf_panel<HostTask> does.  Returns
    (info, piv_tile, piv_off, factored panel)."""
    L = ref_getrf_lib()
    P = np.asfortranarray(np.array(A, dtype=np.float64))
    m = P.shape[0]
    d = min(m, nb)
    pt = np.zeros(max(d, 1), np.int64)
    po = np.zeros(max(d, 1), np.int64)
    info = L.ref_getrf_panel_d(i64(m), i64(nb), i64(nb), _p(P), i64(max(m, 1)), i64(ib), ctypes.c_int(threads),
                               dbl(threshold), _p(pt), _p(po))
    return int(info), pt[:d], po[:d], P


def ref_getrf(A, nb, ib, threshold=1.0, threads=1):
    """Right-looking LU whose panels are SLATE's tile::getrf.  Returns (info,
    piv_tile, piv_off, factors)."""
    L = ref_getrf_lib()
    P = np.asfortranarray(np.array(A, dtype=np.float64))
    m, n = P.shape
    mn = min(m, n)
    pt = np.zeros(max(mn, 1), np.int64)
    po = np.zeros(max(mn, 1), np.int64)
    info = L.ref_getrf_d(i64(m), i64(n), _p(P), i64(max(m, 1)), i64(nb), i64(ib), ctypes.c_int(threads),
                         dbl(threshold), _p(pt), _p(po))
    return int(info), pt[:mn], po[:mn], P


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


def posv_mixed_gmres_nrhs(A, B, nb, itermax=30, tol=0.0, use_fallback=True):
    """posv_mixed_gmres on every column of B (independent FGMRES-IR instances
    sharing one factorisation).  Returns (info, X, iter, per-column iters)."""
    n, nrhs = B.shape
    B = np.asfortranarray(B)
    X = np.zeros((n, nrhs), order="F")
    it = i64(0)
    ci = np.zeros(nrhs, np.int64)
    info = lib().orc_dposv_mixed_gmres_nrhs(i64(n), i64(nrhs), _p(A), i64(n), _p(B), i64(n), _p(X), i64(n),
                                            i64(nb), i64(itermax), dbl(tol), ctypes.c_int(int(use_fallback)),
                                            ctypes.byref(it), _p(ci))
    return int(info), X, int(it.value), ci


def gesv_mixed_gmres_nrhs(A, B, nb, ib=16, itermax=30, tol=0.0, use_fallback=True, panel_threads=1):
    """gesv_mixed_gmres on every column of B.  Returns (info, X, iter,
    per-column iters, pivot tiles, pivot offsets)."""
    n, nrhs = B.shape
    B = np.asfortranarray(B)
    X = np.zeros((n, nrhs), order="F")
    pt = np.zeros(n, np.int64)
    po = np.zeros(n, np.int64)
    it = i64(0)
    ci = np.zeros(nrhs, np.int64)
    info = lib().orc_dgesv_mixed_gmres_nrhs(i64(n), i64(nrhs), _p(A), i64(n), _p(pt), _p(po), _p(B), i64(n),
                                            _p(X), i64(n), i64(nb), i64(ib), ctypes.c_int(panel_threads),
                                            i64(itermax), dbl(tol), ctypes.c_int(int(use_fallback)),
                                            ctypes.byref(it), _p(ci))
    return int(info), X, int(it.value), ci, pt, po


def generate_sigma(n, cond, dist="geo", spd=False, seed=1):
    """Prescribed-spectrum matrix, the CPU statement of the library's device
    generator (same Philox draws; cos/sin may differ in the last bit)."""
    A = np.empty((n, n), order="F")
    lib().orc_dgenerate_sigma(i64(n), dbl(cond), ctypes.c_int({"geo": 0, "logrand": 1}[dist]),
                              ctypes.c_int(int(bool(spd))), i64(seed), _p(A), i64(n))
    return A


# ---------------------------------------------------------------------------
# Random butterfly transforms (src/gerbt.cc, src/internal/Tile_gerbt.hh) and
# gesv_rbt (src/gesv_rbt.cc:100-230), restated with numpy: every product and
# sum is one numpy operation, rounded once, in the order Tile_gerbt.hh writes
# it, so the results are bit-comparable with a kernel that does not fuse.

def rbt_half(n, nb, depth, k):
    """Half length of level k (0 = largest) in elements (gerbt_iterate_1d/_2d:
    half_len = 2^(d-k-1) * ceil(nt / 2^d) tiles of nb)."""
    nt = -(-n // nb)
    inner = -(-nt // (1 << depth))
    return (1 << (depth - k - 1)) * inner * nb


def _halves(n, H):
    x = np.concatenate([np.arange(b, min(b + H, n)) for b in range(0, n, 2 * H)]).astype(np.int64)
    return x[x + H < n], x[x + H >= n]          # paired, unpaired first-half indices


def gerbt2(A, u, v, depth, nb):
    """A <- W_U^T A W_V, levels smallest first (gerbt(U, A, V),
    src/gerbt.cc:160-200; Tile_gerbt.hh:22-80)."""
    A = np.array(A, dtype=np.float64, order="F")
    n = A.shape[0]
    h, r2 = 0.5, 1.0 / np.sqrt(2.0)
    for k in range(depth - 1, -1, -1):
        H = rbt_half(n, nb, depth, k)
        xp, xu = _halves(n, H)
        ix = np.ix_
        a11 = A[ix(xp, xp)].copy(); a12 = A[ix(xp, xp + H)].copy()
        a21 = A[ix(xp + H, xp)].copy(); a22 = A[ix(xp + H, xp + H)].copy()
        s1, s2, d1, d2 = a11 + a12, a21 + a22, a11 - a12, a21 - a22
        u1, u2 = u[xp][:, None], u[xp + H][:, None]
        v1, v2 = v[xp][None, :], v[xp + H][None, :]
        A[ix(xp, xp)] = ((h * u1) * (s1 + s2)) * v1
        A[ix(xp, xp + H)] = ((h * u1) * (d1 + d2)) * v2
        A[ix(xp + H, xp)] = ((h * u2) * (s1 - s2)) * v1
        A[ix(xp + H, xp + H)] = ((h * u2) * (d1 - d2)) * v2
        if len(xu):
            # row unpaired, column paired
            b11 = A[ix(xu, xp)].copy(); b12 = A[ix(xu, xp + H)].copy()
            uu = u[xu][:, None]
            A[ix(xu, xp)] = ((r2 * uu) * (b11 + b12)) * v1
            A[ix(xu, xp + H)] = ((r2 * uu) * (b11 - b12)) * v2
            # row paired, column unpaired
            c11 = A[ix(xp, xu)].copy(); c21 = A[ix(xp + H, xu)].copy()
            vu = v[xu][None, :]
            A[ix(xp, xu)] = ((r2 * u1) * (c11 + c21)) * vu
            A[ix(xp + H, xu)] = ((r2 * u2) * (c11 - c21)) * vu
            # both unpaired
            A[ix(xu, xu)] = (uu * A[ix(xu, xu)]) * vu
    return A


def gerbt1(trans, B, w, depth, nb):
    """B <- W^T B ('T', smallest first) or W B ('N', largest first)
    (gerbt(U, B), src/gerbt.cc:230-280; Tile_gerbt.hh:84-230)."""
    B = np.array(B, dtype=np.float64, order="F")
    n = B.shape[0]
    r2 = 1.0 / np.sqrt(2.0)
    levels = range(depth - 1, -1, -1) if trans == "T" else range(depth)
    for k in levels:
        H = rbt_half(n, nb, depth, k)
        xp, xu = _halves(n, H)
        b1, b2 = B[xp, :].copy(), B[xp + H, :].copy()
        w1, w2 = w[xp][:, None], w[xp + H][:, None]
        if trans == "T":
            B[xp, :] = (r2 * w1) * (b1 + b2)
            B[xp + H, :] = (r2 * w2) * (b1 - b2)
        else:
            B[xp, :] = r2 * ((w1 * b1) + (w2 * b2))
            B[xp + H, :] = r2 * ((w1 * b1) - (w2 * b2))
        if len(xu):
            B[xu, :] = w[xu][:, None] * B[xu, :]
    return B


def gesv_rbt(A, B, nb, u, v, depth=2, ib=16, itermax=30, tol=0.0, use_fallback=True):
    """slate::gesv_rbt with the given diagonals: returns (X, iter, info)
    (src/gesv_rbt.cc:100-230; stopping test internal_util.hh:121-138)."""
    n, nrhs = B.shape
    eps = np.finfo(np.float64).eps
    tol = tol if tol > 0 else eps * np.sqrt(n)
    cte = np.abs(A).sum(1).max() * tol
    Ap = gerbt2(A, u, v, depth, nb)
    info, pt, po, _, _ = getrf(Ap, nb, ib, threshold=0.0)

    def solve(Y):
        Y = gerbt1("T", Y, u, depth, nb)
        getrs(Ap, pt, po, Y, nb)
        return gerbt1("N", Y, v, depth, nb)

    X = np.array(B, order="F")
    if info == 0:
        X = solve(X)
    if itermax == 0:
        return X, 0, info

    def conv(X):
        R = np.asfortranarray(B - A @ X)
        return R, bool(np.all(np.abs(R).max(0) <= np.abs(X).max(0) * cte))

    it = 0
    done = False
    if info == 0:
        R, done = conv(X)
        while not done and it < itermax:
            X = X + solve(R)
            it += 1
            R, done = conv(X)
    if done:
        return X, it, 0
    if use_fallback:
        A2 = np.array(A, order="F")
        X = np.array(B, order="F")
        finfo, _, _ = gesv(A2, X, nb, ib)
        return X, -itermax - 1, finfo
    return X, -itermax - 1, info


def backward_error(A, X, B, sym_lower=False):
    """||B - A X||_1 / (n ||A||_1 ||X||_1), the SLATE tester's check."""
    n, nrhs = X.shape
    A = np.asfortranarray(A)
    X = np.asfortranarray(X)
    B = np.asfortranarray(B)
    return float(lib().orc_backward_error(i64(n), i64(nrhs), _p(A), i64(A.shape[0]),
                                          ctypes.c_int(int(sym_lower)), _p(X), i64(n), _p(B),
                                          i64(n)))
