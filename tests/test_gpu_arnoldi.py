"""Batched CGS2 of the block FGMRES (arnoldi.cu) against numpy.

slt_dcgs2 orthogonalises, for every column of one block-FGMRES step, the new
vector -W(:, i) twice against that column's own basis V_q(:, 0:j) (SLATE's
gemm-based CGS2, src/gesv_mixed_gmres.cc:300-330).  Checked through the C
ABI for columns at different steps j (0 and the last step of a restart
cycle included), slots out of order and a basis store larger than the
active set: the two coefficient vectors, the norm and the resulting vector
agree with the same steps in numpy FP64 to 1e-12 relative (summation order
differs), and the untouched slots are unchanged.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


class Cols(ctypes.Structure):
    _fields_ = [("na", ctypes.c_int), ("q", ctypes.c_int * 16), ("j", ctypes.c_int * 16)]


@pytest.mark.parametrize("n", [1000, 65536 + 17])
def test_cgs2_matches_numpy(slt, n):
    import torch
    L = slt.lib()
    f = L.slt_dcgs2
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.POINTER(Cols), ctypes.c_void_p,
                  ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p]
    wsb = L.slt_cgs_ws_bytes
    wsb.restype = ctypes.c_size_t
    wsb.argtypes = [ctypes.c_int64]
    R1, slots, SC = 31, 16, 4 + 3 * 31
    rng = np.random.default_rng(n)
    Vh = rng.standard_normal((slots, R1, n))
    for q in range(slots):                          # orthonormal bases, as the iteration keeps them
        Q, _ = np.linalg.qr(Vh[q].T)
        Vh[q, :, :] = Q.T
    act = [(5, 0), (0, 3), (11, 29), (2, 7), (15, 1), (7, 12)]
    W = rng.standard_normal((len(act), n))
    dV = torch.from_numpy(Vh.copy()).cuda()
    dW = torch.from_numpy(W.copy()).cuda()
    dS = torch.zeros(slots * SC, dtype=torch.float64, device="cuda")
    ws = torch.empty(wsb(R1), dtype=torch.uint8, device="cuda")
    c = Cols()
    c.na = len(act)
    for i, (q, j) in enumerate(act):
        c.q[i], c.j[i] = q, j
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = f(n, dV.data_ptr(), R1, ctypes.byref(c), dW.data_ptr(), dS.data_ptr(), SC, ws.data_ptr(), s)
    assert rc == 0
    torch.cuda.synchronize()
    V = dV.cpu().numpy()
    S = dS.cpu().numpy()
    for i, (q, j) in enumerate(act):
        B = Vh[q, :j + 1].T
        v = -W[i]
        h = B.T @ v
        v = v - B @ h
        z = B.T @ v
        v = v - B @ z
        nrm = np.linalg.norm(v)
        tol = 1e-12 * np.linalg.norm(W[i])
        assert np.abs(S[q * SC + 4:q * SC + 5 + j] - h).max() <= tol
        assert np.abs(S[q * SC + 4 + R1:q * SC + 5 + R1 + j] - z).max() <= tol
        assert abs(S[q * SC + 3] - nrm) <= tol
        assert np.abs(V[q, j + 1] - v).max() <= tol
        assert np.array_equal(V[q, :j + 1], Vh[q, :j + 1])
    for q in set(range(slots)) - {a for a, _ in act}:
        assert np.array_equal(V[q], Vh[q])


@pytest.mark.parametrize("m", [1000, 70001])
def test_colmax_matches_numpy(slt, m):
    """slt_dcolmax (the residual and solution max-norms of the stopping
    tests): one block per column for short columns, 8192-row segments
    combined by an atomic max for long ones; NaN propagates, -Inf counts as
    Inf, zero columns give 0."""
    import torch
    L = slt.lib()
    f = L.slt_dcolmax
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p]
    n, lda = 6, m + 5
    rng = np.random.default_rng(m)
    A = rng.standard_normal((n, lda))              # column j at A[j, :]
    A[:, m:] = 1e300                               # beyond m: never read
    A[1, m // 2] = np.nan
    A[2, 7] = -np.inf
    A[3, :m] = 0.0
    A[4, m - 1] = -123.0
    dA = torch.from_numpy(A).cuda()
    out = torch.full((n,), -1.0, dtype=torch.float64, device="cuda")
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert f(m, n, dA.data_ptr(), lda, out.data_ptr(), s) == 0
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    ref = np.abs(A[:, :m]).max(axis=1)
    assert np.isnan(got[1]) and np.isinf(got[2]) and got[3] == 0.0
    keep = [0, 4, 5]
    assert np.array_equal(got[keep], ref[keep])
