"""ctypes bindings of the ScaLAPACK-compatible entry points (1 x 1 grid)."""
import ctypes

import numpy as np

c_int_p = ctypes.POINTER(ctypes.c_int)


def ip(x):
    return ctypes.byref(ctypes.c_int(int(x)))


def ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def desc(m, n, mb, lld, dtype=1, rsrc=0, csrc=0):
    """ScaLAPACK's 9-entry descriptor of an m x n matrix on a 1 x 1 grid."""
    return np.array([dtype, 0, m, n, mb, mb, rsrc, csrc, lld], dtype=np.int32)


def call(L, name, *args):
    info = ctypes.c_int(0)
    getattr(L, name)(*args, ctypes.byref(info))
    return info.value


def pdgesv(L, n, nrhs, a, ia, ja, da, ipiv, b, ib, jb, db):
    return call(L, "pdgesv_", ip(n), ip(nrhs), ptr(a), ip(ia), ip(ja), ptr(da), ptr(ipiv), ptr(b), ip(ib), ip(jb),
                ptr(db))
