"""The allocation-free FP64 residual (slt_dresidual_noalloc) against the
allocating entry point (slt_dresidual) and against a host FP64 B - A X,
through the C ABI.

Callers whose device memory belongs to their own pool or to an allocator
that forbids side allocations, or that must not call cudaMalloc where they
need a residual, use the variant whose scratch is a fixed library-owned
device array.  Two calls in a row must each match the allocating residual:
the second call must not see the first call's leftovers in the shared
scratch.  Tolerance: the two entry points may split the columns into
different segments, so sums are compared to 1e-13 relative to
sum_j |A(i,j)| |X(j)| + |B(i)|; the host residual is held to the same bound.
"""
import ctypes

import numpy as np
import pytest

from gpu_util import to_dev, to_host

pytestmark = pytest.mark.gpu

i64, vp, cint = ctypes.c_int64, ctypes.c_void_p, ctypes.c_int


def _entry_points(slt):
    L = slt.lib()
    common = [i64, i64, vp, i64, cint, vp, i64, vp, i64, vp, i64]
    na = L.slt_dresidual_noalloc
    na.argtypes = common + [vp]
    na.restype = cint
    ref = L.slt_dresidual
    ref.argtypes = common + [vp, vp]
    ref.restype = cint
    wsb = L.slt_residual_ws_bytes
    wsb.argtypes = [i64, i64]
    wsb.restype = ctypes.c_size_t
    return na, ref, wsb


def _scale(A, X, B, sym):
    Af = np.tril(A) + np.tril(A, -1).T if sym else A
    return np.abs(Af) @ np.abs(X) + np.abs(B)


@pytest.mark.parametrize("n,nrhs,sym", [(1000, 1, 0), (3000, 5, 1), (2500, 20, 0), (777, 3, 1)])
def test_noalloc_matches_allocating_residual_twice(orc, slt, n, nrhs, sym):
    import torch
    na, ref, wsb = _entry_points(slt)
    s = vp(torch.cuda.current_stream().cuda_stream)
    ws = torch.empty(wsb(n, min(nrhs, 16)), dtype=torch.uint8, device="cuda")
    for call in range(2):
        A = orc.generate(2, 500 + 10 * call + n, n, n)
        X = orc.generate(2, 600 + 10 * call + n, n, nrhs)
        B = orc.generate(2, 700 + 10 * call + n, n, nrhs)
        dA, dX, dB = to_dev(A), to_dev(X), to_dev(B)
        dR1 = to_dev(np.zeros((n, nrhs)))
        dR2 = to_dev(np.zeros((n, nrhs)))
        assert na(n, nrhs, dA.data_ptr(), n, sym, dB.data_ptr(), n, dX.data_ptr(), n, dR1.data_ptr(), n, s) == 0
        # the allocating entry point takes up to 16 right-hand sides per call
        for c0 in range(0, nrhs, 16):
            nc = min(16, nrhs - c0)
            off = 8 * n * c0
            assert ref(n, nc, dA.data_ptr(), n, sym, dB.data_ptr() + off, n, dX.data_ptr() + off, n,
                       dR2.data_ptr() + off, n, vp(ws.data_ptr()), s) == 0
        torch.cuda.synchronize()
        R1, R2 = to_host(dR1), to_host(dR2)
        scale = _scale(A, X, B, sym)
        assert np.all(np.abs(R1 - R2) <= 1e-13 * scale), float(np.max(np.abs(R1 - R2) / scale))
        # independent of the library's kernels: the residual in host FP64
        Af = np.tril(A) + np.tril(A, -1).T if sym else A
        Rh = B - Af @ X
        assert np.all(np.abs(R1 - Rh) <= 1e-13 * scale), float(np.max(np.abs(R1 - Rh) / scale))


def test_noalloc_rejects_oversized_problem_without_launching(slt):
    import torch
    na, _, _ = _entry_points(slt)
    s = vp(torch.cuda.current_stream().cuda_stream)
    n = 2 * 1024 * 1024 // 4 + 1        # n * min(nrhs, 16) just above the 2,097,152 limit
    assert na(n, 4, None, n, 0, None, n, None, n, None, n, s) == -6   # SLT_ERR_LIMIT
