"""Argument and descriptor checks of the ScaLAPACK-compatible entry points:
they run on the host before any device work, so they need no GPU.  A bad
entry k of descriptor argument p gives info = -(100 p + k); a submatrix that
does not fit gives -(position of ia or ja); a bad scalar gives -(position)."""
import ctypes

import numpy as np
import pytest

from scalapack_util import call, desc, ip, pdgesv, ptr


@pytest.fixture(scope="module")
def L():
    from slate_gb300 import LIB_PATH
    return ctypes.CDLL(LIB_PATH)


def _arrays(n=8, nrhs=2):
    a = np.asfortranarray(np.eye(n))
    b = np.asfortranarray(np.ones((n, nrhs)))
    return a, b, np.zeros(n, np.int32)


@pytest.mark.parametrize("bad,code", [
    (dict(dtype=2), -601), (dict(rsrc=1), -607), (dict(csrc=1), -608), (dict(lld=4), -609)])
def test_pdgesv_bad_desca(L, bad, code):
    n = 8
    a, b, piv = _arrays(n)
    kw = dict(lld=n)
    kw.update(bad)
    da = desc(n, n, 4, **kw)
    db = desc(n, 2, 4, n)
    assert pdgesv(L, n, 2, a, 1, 1, da, piv, b, 1, 1, db) == code


def test_pdgesv_bad_scalars_and_offsets(L):
    n = 8
    a, b, piv = _arrays(n)
    da, db = desc(n, n, 4, n), desc(n, 2, 4, n)
    assert pdgesv(L, -1, 2, a, 1, 1, da, piv, b, 1, 1, db) == -1
    assert pdgesv(L, n, -1, a, 1, 1, da, piv, b, 1, 1, db) == -2
    assert pdgesv(L, n, 2, a, 2, 1, da, piv, b, 1, 1, db) == -4      # ia + n - 1 > M
    assert pdgesv(L, n, 2, a, 1, 0, da, piv, b, 1, 1, db) == -5
    assert pdgesv(L, n, 2, a, 1, 1, da, piv, b, 1, 2, db) == -10     # jb + nrhs - 1 > N_B
    assert pdgesv(L, n, 2, a, 1, 1, da, piv, b, 1, 1, desc(n, 2, 0, n)) == -1105   # MB < 1
    assert pdgesv(L, 0, 2, a, 1, 1, da, piv, b, 1, 1, db) == 0       # quick return


def test_other_entry_points_check_arguments(L):
    n = 6
    a, b, piv = _arrays(n)
    da, db = desc(n, n, 4, n), desc(n, 2, 4, n)
    bad = desc(n, n, 4, n, dtype=7)
    assert call(L, "pdgetrf_", ip(n), ip(n), ptr(a), ip(1), ip(1), ptr(bad), ptr(piv)) == -601
    assert call(L, "pdgetrs_", b"X", ip(n), ip(2), ptr(a), ip(1), ip(1), ptr(da), ptr(piv), ptr(b), ip(1), ip(1),
                ptr(db)) == -1
    assert call(L, "pdgetrs_", b"N", ip(n), ip(2), ptr(a), ip(1), ip(1), ptr(bad), ptr(piv), ptr(b), ip(1), ip(1),
                ptr(db)) == -701
    assert call(L, "pdposv_", b"Q", ip(n), ip(2), ptr(a), ip(1), ip(1), ptr(da), ptr(b), ip(1), ip(1), ptr(db)) == -1
    assert call(L, "pdpotrf_", b"L", ip(n), ptr(a), ip(1), ip(1), ptr(bad)) == -601
    assert call(L, "pdpotrs_", b"L", ip(n), ip(2), ptr(a), ip(1), ip(1), ptr(da), ptr(b), ip(1), ip(1),
                ptr(bad)) == -1101
    assert call(L, "pdpotri_", b"U", ip(n), ptr(a), ip(3), ip(1), ptr(da)) == -4
    x = np.zeros_like(b)
    it = ctypes.c_int(0)
    assert call(L, "pdsgesv_", ip(n), ip(2), ptr(a), ip(1), ip(1), ptr(da), ptr(piv), ptr(b), ip(1), ip(1), ptr(db),
                ptr(x), ip(1), ip(1), ptr(bad), ctypes.byref(it)) == -1501
    # workspace queries of getri / gecon return size 1 without touching A
    work = np.zeros(1)
    iwork = np.zeros(1, np.int32)
    assert call(L, "pdgetri_", ip(n), ptr(a), ip(1), ip(1), ptr(da), ptr(piv), ptr(work), ip(-1), ptr(iwork),
                ip(-1)) == 0
    assert work[0] == 1.0 and iwork[0] == 1
    an = ctypes.c_double(1.0)
    rc = ctypes.c_double(0.0)
    assert call(L, "pdgecon_", b"1", ip(-1), ptr(a), ip(1), ip(1), ptr(da), ctypes.byref(an), ctypes.byref(rc),
                ptr(work), ip(1), ptr(iwork), ip(1)) == -2
