"""slate_gb300 -- GB300-native LU / Cholesky solve path with SLATE's API.

Python mirror of SLATE's drivers for one GPU (a 1 x 1 grid with
Target::Devices): ``getrf/getrs/gesv``, ``potrf/potrs/posv``, ``gesv_mixed``,
``gesv_mixed_gmres``, ``posv_mixed`` and ``posv_mixed_gmres``, plus the
LAPACK-compatible host entry points (``lapack`` namespace).  Every call goes
through the C ABI of ``libslate_gb300.so`` (include/slate_gb300.h); there is
no CPU or library fallback -- importing fails if the library is missing.

Device arrays are torch CUDA tensors in column-major layout (``colmajor()``
makes one); host arrays for the LAPACK entry points are Fortran-ordered numpy
arrays.
"""
import ctypes
import os
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libslate_gb300.so")

PREC_FP64, PREC_FP32, PREC_TF32, PREC_BF16, PREC_FP16 = 0, 1, 2, 3, 4
_PREC_NAMES = {"fp64": 0, "fp32": 1, "tf32": 2, "bf16": 3, "fp16": 4, "fp8": 5, "tf32x3": 6}
_REFINE_NAMES = {"ir": 0, "gmres": 1, "ir+gmres": 2}


class SlateError(RuntimeError):
    """A non-zero status from the library (slate::Exception analogue)."""


class _Options(ctypes.Structure):
    _fields_ = [("nb", ctypes.c_int64), ("ib", ctypes.c_int64), ("lookahead", ctypes.c_int64),
                ("max_iterations", ctypes.c_int64), ("tolerance", ctypes.c_double),
                ("use_fallback", ctypes.c_int), ("pivot_threshold", ctypes.c_double),
                ("factor_precision", ctypes.c_int), ("gemm_engine", ctypes.c_int),
                ("refine", ctypes.c_int), ("equilibrate", ctypes.c_int), ("lo_retry", ctypes.c_int),
                ("depth", ctypes.c_int64), ("method_lu", ctypes.c_int), ("residual_engine", ctypes.c_int)]


@dataclass
class Options:
    """SLATE Option keys used on this path (include/slate/enums.hh:453-490)."""
    nb: int = 512
    ib: int = 32
    lookahead: int = 1
    max_iterations: int = 30
    tolerance: float = 0.0
    use_fallback: bool = True
    pivot_threshold: float = 1.0
    factor_precision: object = "fp32"
    gemm_engine: int = 0
    refine: object = "ir"          # "ir" (SLATE's IR), "gmres" (FGMRES-IR) or "ir+gmres" (GMRES-IR once IR stalls)
    equilibrate: int = -1          # -1 auto (on for bf16/fp16), 0 off, 1 on
    lo_retry: int = -1             # -1 auto (on for bf16/fp16): FP32 retry before the FP64 fallback
    depth: int = 2                 # Option::Depth of gesv_rbt's butterflies
    method_lu: str = "P"           # Option::MethodLU: "P" partial pivoting, "N" none, "C" CALU
    residual_engine: int = 0       # FP64 residuals: 0 auto, 1 FP64 FMA, 2 tensor cores (digit splitting)

    def _c(self):
        p = self.factor_precision
        p = _PREC_NAMES[p] if isinstance(p, str) else int(p)
        return _Options(int(self.nb), int(self.ib), int(self.lookahead), int(self.max_iterations),
                        float(self.tolerance), int(bool(self.use_fallback)),
                        float(self.pivot_threshold), p, int(self.gemm_engine),
                        _REFINE_NAMES[self.refine] if isinstance(self.refine, str) else int(self.refine),
                        int(self.equilibrate), int(self.lo_retry), int(self.depth),
                        ord(self.method_lu[0]) if isinstance(self.method_lu, str) else int(self.method_lu),
                        int(self.residual_engine))


_lib = None


def lib():
    """Load libslate_gb300.so; raise if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libslate_gb300.so not built: run python -m slate_gb300.build")
        L = ctypes.CDLL(LIB_PATH)
        i64, vp, ip, dp = ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64)
        optp = ctypes.POINTER(_Options)
        iptr = ctypes.POINTER(ctypes.c_int)
        sig = {
            "slt_dgetrf_device": [i64, i64, vp, i64, ip, optp, vp, dp],
            "slt_sgetrf_device": [i64, i64, vp, i64, ip, optp, vp, dp],
            "slt_dgetrs_device": [i64, i64, vp, i64, ip, vp, i64, optp, vp],
            "slt_sgetrs_device": [i64, i64, vp, i64, ip, vp, i64, optp, vp],
            "slt_dgesv_device": [i64, i64, vp, i64, ip, vp, i64, optp, vp, dp],
            "slt_dpotrf_device": [i64, vp, i64, optp, vp, dp],
            "slt_spotrf_device": [i64, vp, i64, optp, vp, dp],
            "slt_dpotrs_device": [i64, i64, vp, i64, vp, i64, optp, vp],
            "slt_dposv_device": [i64, i64, vp, i64, vp, i64, optp, vp, dp],
            "slt_dsgesv_device": [i64, i64, vp, i64, ip, vp, i64, vp, i64, optp, vp, iptr, dp],
            "slt_dgesv_rbt_device": [i64, i64, vp, i64, vp, i64, vp, i64, optp, vp, iptr, dp],
            "slt_dsgesv_gmres_device": [i64, i64, vp, i64, ip, vp, i64, vp, i64, optp, vp, iptr, dp],
            "slt_dsposv_device": [i64, i64, vp, i64, vp, i64, vp, i64, optp, vp, iptr, dp],
            "slt_dsposv_gmres_device": [i64, i64, vp, i64, vp, i64, vp, i64, optp, vp, iptr, dp],
            "slt_dgenerate_device": [ctypes.c_int, i64, i64, i64, i64, i64, vp, i64, vp],
        }
        for name, args in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = ctypes.c_int
        L.slt_status_string.restype = ctypes.c_char_p
        L.slt_status_string.argtypes = [ctypes.c_int]
        L.slt_version.restype = ctypes.c_char_p
        L.slt_timer.restype = ctypes.c_double
        L.slt_timer.argtypes = [ctypes.c_char_p]
        _lib = L
    return _lib


def version():
    return lib().slt_version().decode()


def timer(name):
    """Seconds of a named phase of the last driver call (slate::timers key)."""
    return float(lib().slt_timer(name.encode()))


def _check(rc):
    if rc != 0:
        raise SlateError("slate_gb300: %s (status %d)" % (lib().slt_status_string(rc).decode(), rc))


# ---------------------------------------------------------------------------
# torch device helpers
def colmajor(x):
    """Return a column-major (Fortran-strided) copy/view of a 2-D tensor."""
    if x.dim() == 1:
        x = x.reshape(-1, 1)
    if x.stride(0) == 1 and (x.shape[1] <= 1 or x.stride(1) >= max(1, x.shape[0])):
        return x
    return x.t().contiguous().t()


def _ld(x):
    return max(1, x.stride(1) if x.shape[1] > 1 else x.shape[0])


def _dev(x, dtype=None):
    import torch
    if not (isinstance(x, torch.Tensor) and x.is_cuda):
        raise TypeError("expected a CUDA tensor")
    if dtype is not None and x.dtype != dtype:
        raise TypeError("expected dtype %s, got %s" % (dtype, x.dtype))
    if x.dim() != 2 or (x.stride(0) != 1 and x.shape[0] > 1):
        raise ValueError("expected a column-major 2-D tensor (use slate_gb300.colmajor)")
    return ctypes.c_void_p(x.data_ptr())


def _stream():
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _opts(opts):
    o = opts if isinstance(opts, Options) else Options(**(opts or {}))
    return ctypes.byref(o._c()), o


def _prefix(t):
    """SLATE's precision letter of a tensor: s, d, c (complex<float>) or z."""
    import torch
    p = {torch.float32: "s", torch.float64: "d", torch.complex64: "c", torch.complex128: "z"}.get(t.dtype)
    if p is None:
        raise TypeError("unsupported dtype %s" % t.dtype)
    return p


_I64, _VP, _OPTP = ctypes.c_int64, ctypes.c_void_p, ctypes.POINTER(_Options)
_DP = ctypes.POINTER(ctypes.c_int64)
_SIGS = {
    "getrf": [_I64, _I64, _VP, _I64, _VP, _OPTP, _VP, _DP],
    "getrs_c": [ctypes.c_char, _I64, _I64, _VP, _I64, _VP, _VP, _I64, _OPTP, _VP],
    "gesv": [_I64, _I64, _VP, _I64, _VP, _VP, _I64, _OPTP, _VP, _DP],
    "potrf": [_I64, _VP, _I64, _OPTP, _VP, _DP],
    "potrs": [_I64, _I64, _VP, _I64, _VP, _I64, _OPTP, _VP],
    "posv": [_I64, _I64, _VP, _I64, _VP, _I64, _OPTP, _VP, _DP],
}


def _entry(name, sig):
    f = getattr(lib(), name)
    f.argtypes = _SIGS[sig]
    f.restype = ctypes.c_int
    return f


def _ipiv_buf(n, device):
    import torch
    return torch.zeros(max(n, 1), dtype=torch.int32, device=device)


# ---------------------------------------------------------------------------
# SLATE drivers (include/slate/slate.hh:503-770)
def getrf(A, opts=None):
    """LU with partial pivoting in place (slate::getrf), float32 / float64 /
    complex64 / complex128.  Returns (info, ipiv) with ipiv per panel (row of
    panel k relative to row k*nb)."""
    po, o = _opts(opts)
    m, n = A.shape
    ipiv = _ipiv_buf(min(m, n), A.device)
    info = ctypes.c_int64(0)
    f = _entry("slt_%sgetrf_device" % _prefix(A), "getrf")
    _check(f(m, n, _dev(A), _ld(A), ctypes.c_void_p(ipiv.data_ptr()), po, _stream(), ctypes.byref(info)))
    return int(info.value), ipiv[:min(m, n)]


def getrs(A, ipiv, B, opts=None, trans="N"):
    """Solve op(A) X = B with the factors of getrf, op = trans ('N', 'T' or
    'C'); B is overwritten (slate::getrs)."""
    po, o = _opts(opts)
    n = A.shape[0]
    p = _prefix(A)
    t = trans.upper()
    if p in "cz":
        f = _entry("slt_%sgetrs_device" % p, "getrs_c")
        _check(f(t.encode(), n, B.shape[1], _dev(A), _ld(A), ctypes.c_void_p(ipiv.data_ptr()), _dev(B), _ld(B), po,
                 _stream()))
        return
    if t != "N":
        f = _entry("slt_%sgetrs_trans_device" % p, "getrs_c")
        _check(f(t.encode(), n, B.shape[1], _dev(A), _ld(A), ctypes.c_void_p(ipiv.data_ptr()), _dev(B), _ld(B), po,
                 _stream()))
        return
    f = lib().slt_dgetrs_device if p == "d" else lib().slt_sgetrs_device
    _check(f(n, B.shape[1], _dev(A), _ld(A), ctypes.c_void_p(ipiv.data_ptr()), _dev(B), _ld(B), po,
             _stream()))


def gecondest(LU, ipiv, anorm, norm="1", opts=None):
    """slate::gecondest: reciprocal condition number estimate from getrf's
    factors; anorm = ||A|| in `norm` ('1' or 'I')."""
    po, o = _opts(opts)
    f = lib().slt_dgecondest_device
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_char, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_double,
                  ctypes.POINTER(ctypes.c_double), ctypes.POINTER(_Options), ctypes.c_void_p]
    r = ctypes.c_double(0.0)
    _check(f(norm.encode(), LU.shape[0], _dev(LU), _ld(LU), ctypes.c_void_p(ipiv.data_ptr()), float(anorm),
             ctypes.byref(r), po, _stream()))
    return r.value


def pocondest(L, anorm, norm="1", opts=None):
    """slate::pocondest: reciprocal condition number estimate from potrf's
    lower factor; anorm = ||A||."""
    po, o = _opts(opts)
    f = lib().slt_dpocondest_device
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_char, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_double,
                  ctypes.POINTER(ctypes.c_double), ctypes.POINTER(_Options), ctypes.c_void_p]
    r = ctypes.c_double(0.0)
    _check(f(norm.encode(), L.shape[0], _dev(L), _ld(L), float(anorm), ctypes.byref(r), po, _stream()))
    return r.value


def gesv(A, B, opts=None):
    """slate::gesv: A <- LU, B <- X.  Returns (info, ipiv)."""
    po, o = _opts(opts)
    n = A.shape[0]
    p = _prefix(A)
    if p == "s":
        info, ipiv = getrf(A, opts)
        if info == 0:
            getrs(A, ipiv, B, opts)
        return info, ipiv
    ipiv = _ipiv_buf(n, A.device)
    info = ctypes.c_int64(0)
    f = _entry("slt_%sgesv_device" % p, "gesv")
    _check(f(n, B.shape[1], _dev(A), _ld(A), ctypes.c_void_p(ipiv.data_ptr()), _dev(B, A.dtype), _ld(B), po,
             _stream(), ctypes.byref(info)))
    return int(info.value), ipiv[:n]


def potrf(A, opts=None):
    """Cholesky A = L L^H of the lower triangle in place (slate::potrf).  Returns info."""
    po, o = _opts(opts)
    info = ctypes.c_int64(0)
    f = _entry("slt_%spotrf_device" % _prefix(A), "potrf")
    _check(f(A.shape[0], _dev(A), _ld(A), po, _stream(), ctypes.byref(info)))
    return int(info.value)


def potrs(A, B, opts=None):
    """slate::potrs with potrf's lower factor; B <- X."""
    po, o = _opts(opts)
    f = _entry("slt_%spotrs_device" % _prefix(A), "potrs")
    _check(f(A.shape[0], B.shape[1], _dev(A), _ld(A), _dev(B, A.dtype), _ld(B), po, _stream()))


def posv(A, B, opts=None):
    """slate::posv (lower): A <- L, B <- X.  Returns info."""
    po, o = _opts(opts)
    info = ctypes.c_int64(0)
    f = _entry("slt_%sposv_device" % _prefix(A), "posv")
    _check(f(A.shape[0], B.shape[1], _dev(A), _ld(A), _dev(B, A.dtype), _ld(B), po, _stream(), ctypes.byref(info)))
    return int(info.value)


def _mixed(fn, chol, A, B, X, opts):
    import torch
    po, o = _opts(opts)
    n = A.shape[0]
    info = ctypes.c_int64(0)
    it = ctypes.c_int(0)
    args = [n, B.shape[1], _dev(A, torch.float64), _ld(A)]
    ipiv = None
    if not chol:
        ipiv = _ipiv_buf(n, A.device)
        args.append(ctypes.c_void_p(ipiv.data_ptr()))
    args += [_dev(B, torch.float64), _ld(B), _dev(X, torch.float64), _ld(X), po, _stream(),
             ctypes.byref(it), ctypes.byref(info)]
    _check(fn(*args))
    return int(info.value), int(it.value), (ipiv[:n] if ipiv is not None else None)


def gesv_mixed(A, B, X, opts=None):
    """slate::gesv_mixed: low-precision LU + FP64 iterative refinement
    (complex128: gesv_mixed<complex<double>, complex<float>>, zcgesv).
    Returns (info, iter, ipiv)."""
    import torch
    if A.dtype == torch.complex128:
        po, o = _opts(opts)
        n = A.shape[0]
        info = ctypes.c_int64(0)
        it = ctypes.c_int(0)
        ipiv = _ipiv_buf(n, A.device)
        f = lib().slt_zcgesv_device
        f.restype = ctypes.c_int
        _check(f(ctypes.c_int64(n), ctypes.c_int64(B.shape[1]), _dev(A), ctypes.c_int64(_ld(A)),
                 ctypes.c_void_p(ipiv.data_ptr()), _dev(B, A.dtype), ctypes.c_int64(_ld(B)), _dev(X, A.dtype),
                 ctypes.c_int64(_ld(X)), po, _stream(), ctypes.byref(it), ctypes.byref(info)))
        return int(info.value), int(it.value), ipiv[:n]
    return _mixed(lib().slt_dsgesv_device, False, A, B, X, opts)


def gesv_mixed_gmres(A, B, X, opts=None):
    """slate::gesv_mixed_gmres: low-precision LU + FP64 FGMRES-IR."""
    return _mixed(lib().slt_dsgesv_gmres_device, False, A, B, X, opts)


def gesv_rbt(A, B, X, opts=None):
    """slate::gesv_rbt: random butterfly transform, LU without pivoting, FP64
    refinement (src/gesv_rbt.cc).  A receives the factors of the transformed
    matrix.  Returns (info, iter)."""
    import torch
    po, o = _opts(opts)
    info = ctypes.c_int64(0)
    it = ctypes.c_int(0)
    _check(lib().slt_dgesv_rbt_device(A.shape[0], B.shape[1], _dev(A, torch.float64), _ld(A),
                                      _dev(B, torch.float64), _ld(B), _dev(X, torch.float64), _ld(X), po,
                                      _stream(), ctypes.byref(it), ctypes.byref(info)))
    return int(info.value), int(it.value)


def _vec(w, n):
    import torch
    if not (isinstance(w, torch.Tensor) and w.is_cuda and w.dtype == torch.float64 and w.is_contiguous()
            and w.numel() >= n):
        raise TypeError("expected a contiguous float64 CUDA vector of at least %d entries" % n)
    return ctypes.c_void_p(w.data_ptr())


def gerbt2(A, u, v, depth, nb):
    """slate::gerbt(U, A, V): A <- W_U^T A W_V with diagonals u, v (n)."""
    import torch
    L = lib()
    L.slt_dgerbt2_device.argtypes = [ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                     ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p]
    _check(L.slt_dgerbt2_device(A.shape[0], _dev(A, torch.float64), _ld(A), _vec(u, A.shape[0]),
                                _vec(v, A.shape[0]), int(depth), int(nb), _stream()))


def gerbt1(trans, B, w, depth, nb):
    """slate::gerbt(U, B): B <- W^T B (trans 'T') or W B ('N')."""
    import torch
    L = lib()
    L.slt_dgerbt1_device.argtypes = [ctypes.c_char, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p,
                                     ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                     ctypes.c_void_p]
    _check(L.slt_dgerbt1_device(trans.encode() if isinstance(trans, str) else trans, B.shape[0], B.shape[1],
                                _dev(B, torch.float64), _ld(B), _vec(w, B.shape[0]), int(depth), int(nb),
                                _stream()))


def rbt_diag(n, seed, device="cuda"):
    """The random butterfly diagonal exp(r / 20), r uniform(-1, 1) (Philox)."""
    import torch
    w = torch.empty(n, dtype=torch.float64, device=device)
    L = lib()
    L.slt_drbt_diag_device.argtypes = [ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p]
    _check(L.slt_drbt_diag_device(int(n), int(seed), ctypes.c_void_p(w.data_ptr()), _stream()))
    return w


def posv_mixed(A, B, X, opts=None):
    """slate::posv_mixed (A lower).  Returns (info, iter, None)."""
    return _mixed(lib().slt_dsposv_device, True, A, B, X, opts)


def posv_mixed_gmres(A, B, X, opts=None):
    return _mixed(lib().slt_dsposv_gmres_device, True, A, B, X, opts)


def generate(dist, seed, A, ioff=0, joff=0):
    """slate::random::generate on the device (matgen/random.cc)."""
    _check(lib().slt_dgenerate_device(int(dist), int(seed), A.shape[0], A.shape[1], ioff, joff,
                                      _dev(A), _ld(A), _stream()))


def generate_sigma(A, cond, dist="geo", spd=False, seed=1):
    """Prescribed-spectrum test matrix on the device: A = Q1 diag(sigma) Q2^T,
    or Q diag(sigma) Q^T when spd, with SLATE's "geo" / "logrand" sigma of
    condition number cond (matgen/generate_sigma.hh:73-125)."""
    f = lib().slt_dgenerate_sigma
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int64, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int64, ctypes.c_void_p,
                  ctypes.c_int64, ctypes.c_void_p]
    _check(f(A.shape[0], float(cond), {"geo": 0, "logrand": 1}[dist], int(bool(spd)), int(seed), _dev(A), _ld(A),
             _stream()))


class VBatch:
    """Device descriptor arrays of a variable-size batch.

    systems: list of (kind, A, B) with kind 0 (general, LU) or 1 (SPD,
    Cholesky, lower triangle used), A an n x n and B an n x nrhs
    column-major float64 CUDA tensor (see colmajor).  X: optional list of
    solution tensors shaped like B (mixed solver).  The pointer arrays refer
    to the caller's tensors, which must outlive the call."""

    def __init__(self, systems, X=None):
        import torch
        dev = systems[0][1].device if systems else torch.device("cuda")
        i32 = dict(dtype=torch.int32, device=dev)
        i64 = dict(dtype=torch.int64, device=dev)
        self.batch = len(systems)
        self.kind = torch.tensor([k for k, _, _ in systems], **i32)
        self.n = torch.tensor([a.shape[0] for _, a, _ in systems], **i32)
        self.nrhs = torch.tensor([b.shape[1] for _, _, b in systems], **i32)
        self.lda = torch.tensor([_ld(a) for _, a, _ in systems], **i32)
        self.ldb = torch.tensor([_ld(b) for _, _, b in systems], **i32)
        self.A = torch.tensor([a.data_ptr() for _, a, _ in systems], **i64)
        self.B = torch.tensor([b.data_ptr() for _, _, b in systems], **i64)
        self.ipiv_t = [torch.zeros(max(1, a.shape[0]), **i32) if k == 0 else None for k, a, _ in systems]
        self.ipiv = torch.tensor([p.data_ptr() if p is not None else 0 for p in self.ipiv_t], **i64)
        self.info = torch.zeros(self.batch, **i32)
        self.iter = torch.zeros(self.batch, **i32)
        if X is not None:
            self.X = torch.tensor([x.data_ptr() for x in X], **i64)
            self.ldx = torch.tensor([_ld(x) for x in X], **i32)


def solve_vbatched(vb):
    """FP64 variable-size batched gesv/posv: A <- factors, B <- X.
    Returns the info array (CPU numpy)."""
    f = lib().slt_dsolve_vbatched
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int64] + [ctypes.c_void_p] * 9 + [ctypes.c_void_p]
    _check(f(vb.batch, vb.kind.data_ptr(), vb.n.data_ptr(), vb.nrhs.data_ptr(), vb.A.data_ptr(),
             vb.lda.data_ptr(), vb.ipiv.data_ptr(), vb.B.data_ptr(), vb.ldb.data_ptr(), vb.info.data_ptr(),
             _stream()))
    return vb.info.cpu().numpy()


def solve_mixed_vbatched(vb, opts=None):
    """Mixed variable-size batched solve (FP32 factors + FP64 refinement).
    Returns (info, iter) as CPU numpy arrays."""
    o = opts or Options()
    f = lib().slt_dsolve_mixed_vbatched
    f.restype = ctypes.c_int
    f.argtypes = ([ctypes.c_int64] + [ctypes.c_void_p] * 12 + [ctypes.c_int64, ctypes.c_double, ctypes.c_int,
                                                               ctypes.c_void_p])
    _check(f(vb.batch, vb.kind.data_ptr(), vb.n.data_ptr(), vb.nrhs.data_ptr(), vb.A.data_ptr(),
             vb.lda.data_ptr(), vb.ipiv.data_ptr(), vb.B.data_ptr(), vb.ldb.data_ptr(), vb.X.data_ptr(),
             vb.ldx.data_ptr(), vb.iter.data_ptr(), vb.info.data_ptr(), int(o.max_iterations),
             float(o.tolerance), int(bool(o.use_fallback)), _stream()))
    return vb.info.cpu().numpy(), vb.iter.cpu().numpy()


def ipiv_to_lapack(ipiv, nb):
    """Per-panel pivots -> LAPACK 1-based ipiv (lapack_api/lapack_gesv.cc:90-100)."""
    p = np.asarray(ipiv.cpu() if hasattr(ipiv, "cpu") else ipiv, dtype=np.int64)
    r = np.arange(p.size)
    return (r // nb) * nb + p + 1


# ---------------------------------------------------------------------------
# LAPACK-compatible host entry points (lapack_api/*.cc)
class lapack:
    @staticmethod
    def _ptr(a):
        return a.ctypes.data_as(ctypes.c_void_p)

    @staticmethod
    def dgesv(a, b):
        """slate_dgesv: returns (info, ipiv); a <- LU, b <- X (Fortran arrays)."""
        n, nrhs = a.shape[0], b.shape[1]
        ipiv = np.zeros(n, np.int32)
        info = ctypes.c_int(0)
        c = ctypes.c_int
        lib().slate_dgesv(ctypes.byref(c(n)), ctypes.byref(c(nrhs)), lapack._ptr(a), ctypes.byref(c(n)),
                          lapack._ptr(ipiv), lapack._ptr(b), ctypes.byref(c(n)), ctypes.byref(info))
        return info.value, ipiv

    @staticmethod
    def dgetrf(a):
        m, n = a.shape
        ipiv = np.zeros(min(m, n), np.int32)
        info = ctypes.c_int(0)
        c = ctypes.c_int
        lib().slate_dgetrf(ctypes.byref(c(m)), ctypes.byref(c(n)), lapack._ptr(a), ctypes.byref(c(m)),
                           lapack._ptr(ipiv), ctypes.byref(info))
        return info.value, ipiv

    @staticmethod
    def dgetrs(a, ipiv, b):
        n, nrhs = a.shape[0], b.shape[1]
        info = ctypes.c_int(0)
        c = ctypes.c_int
        ipiv = np.ascontiguousarray(ipiv, dtype=np.int32)
        lib().slate_dgetrs(ctypes.c_char_p(b"N"), ctypes.byref(c(n)), ctypes.byref(c(nrhs)), lapack._ptr(a),
                           ctypes.byref(c(n)), lapack._ptr(ipiv), lapack._ptr(b), ctypes.byref(c(n)),
                           ctypes.byref(info))
        return info.value

    @staticmethod
    def dsgesv(a, b, x):
        n, nrhs = a.shape[0], b.shape[1]
        ipiv = np.zeros(n, np.int32)
        info = ctypes.c_int(0)
        it = ctypes.c_int(0)
        c = ctypes.c_int
        lib().slate_dsgesv(ctypes.byref(c(n)), ctypes.byref(c(nrhs)), lapack._ptr(a), ctypes.byref(c(n)),
                           lapack._ptr(ipiv), lapack._ptr(b), ctypes.byref(c(n)), lapack._ptr(x),
                           ctypes.byref(c(n)), None, None, ctypes.byref(it), ctypes.byref(info))
        return info.value, it.value, ipiv

    @staticmethod
    def dposv(uplo, a, b):
        n, nrhs = a.shape[0], b.shape[1]
        info = ctypes.c_int(0)
        c = ctypes.c_int
        lib().slate_dposv(ctypes.c_char_p(uplo.encode()), ctypes.byref(c(n)), ctypes.byref(c(nrhs)),
                          lapack._ptr(a), ctypes.byref(c(n)), lapack._ptr(b), ctypes.byref(c(n)),
                          ctypes.byref(info))
        return info.value

    @staticmethod
    def dpotrf(uplo, a):
        n = a.shape[0]
        info = ctypes.c_int(0)
        c = ctypes.c_int
        lib().slate_dpotrf(ctypes.c_char_p(uplo.encode()), ctypes.byref(c(n)), lapack._ptr(a),
                           ctypes.byref(c(n)), ctypes.byref(info))
        return info.value
