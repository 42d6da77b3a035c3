"""One-launch triangular sweeps (slt_ssweep / slt_dsweep) against scipy's
solve_triangular in float64 on the same (rounded) triangle.

The six kinds are the triangles getrs / potrs solve with: 0 unit lower,
1 upper, 2 lower, 3 lower^T, 4 upper^T, 5 unit lower^T.  Triangles are
diagonally dominant (off-diagonal entries U(-1, 1) / n), so the solution is
well conditioned and the sweep must match to a few units of its working
precision: relative error <= 2e-5 (float) / 1e-12 (double).  Sizes cover a
single row, exact and ragged multiples of the 64-row block, right-hand-side
counts on both sides of the 4-column split, padded leading dimensions,
back-to-back launches on one scratch buffer and every cluster size of the
FP32 16-right-hand-side sweep.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KINDS = {0: ("L", "N", True), 1: ("U", "N", False), 2: ("L", "N", False),
         3: ("L", "T", False), 4: ("U", "T", False), 5: ("L", "T", True)}
TOL = {np.float32: 2e-5, np.float64: 1e-12}


def _triangle(n, lower, seed, dtype):
    rng = np.random.default_rng(seed)
    M = rng.uniform(-1, 1, (n, n)) / max(n, 1)
    M[np.diag_indices(n)] = 1.0 + rng.uniform(0, 1, n)
    if lower:
        M = np.tril(M)
    else:
        M = np.triu(M)
    # the untouched triangle holds noise the sweep must ignore
    noise = rng.uniform(-5, 5, (n, n))
    M = M + (np.triu(noise, 1) if lower else np.tril(noise, -1))
    return M.astype(dtype).astype(np.float64)


def _sweep(slt, torch, kind, M, B, dtype, ldm_pad=0, ldx_pad=0, flags=None):
    n, nrhs = B.shape
    tdt = torch.float32 if dtype == np.float32 else torch.float64
    # column-major with leading dimensions n + pad
    Mst = torch.zeros(n, n + ldm_pad, dtype=tdt, device="cuda")
    Mst[:, :n] = torch.from_numpy(np.ascontiguousarray(M.T)).to(tdt).cuda()
    Xst = torch.zeros(nrhs, n + ldx_pad, dtype=tdt, device="cuda")
    Xst[:, :n] = torch.from_numpy(np.ascontiguousarray(B.T)).to(tdt).cuda()
    L = slt.lib()
    L.slt_sweep_flags_bytes.restype = ctypes.c_size_t
    L.slt_sweep_flags_bytes.argtypes = [ctypes.c_int64]
    if flags is None:
        flags = torch.full((L.slt_sweep_flags_bytes(n),), 0xA5, dtype=torch.uint8, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    f = L.slt_ssweep if dtype == np.float32 else L.slt_dsweep
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                  ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = f(kind, n, nrhs, Mst.data_ptr(), n + ldm_pad, Xst.data_ptr(), n + ldx_pad, flags.data_ptr(),
           status.data_ptr(), s)
    assert rc == 0, rc
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    return Xst[:, :n].double().cpu().numpy().T, flags


def _reference(kind, M, B):
    from scipy.linalg import solve_triangular
    uplo, trans, unit = KINDS[kind]
    return solve_triangular(M, B, lower=(uplo == "L"), trans=trans, unit_diagonal=unit)


# (> 4 right-hand sides in FP32 take the cp.async / register-tile kernel:
#  16-byte copies when the leading dimension allows, 4-byte copies otherwise)
CASES = [(1, 1), (64, 4), (65, 3), (200, 1), (1000, 5), (4100, 4), (777, 16), (4100, 16), (999, 16), (130, 8)]


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("kind", sorted(KINDS))
@pytest.mark.parametrize("n,nrhs", CASES)
def test_sweep_matches_scipy(slt, kind, dtype, n, nrhs):
    import torch
    uplo, _, _ = KINDS[kind]
    M = _triangle(n, uplo == "L", 100 * kind + n, dtype)
    B = np.random.default_rng(n + nrhs).uniform(-1, 1, (n, nrhs)).astype(dtype).astype(np.float64)
    X, _ = _sweep(slt, torch, kind, M, B, dtype, ldm_pad=3 if n % 2 else 0, ldx_pad=1)
    Xr = _reference(kind, M, B)
    err = np.abs(X - Xr).max() / max(np.abs(Xr).max(), 1e-300)
    assert err <= TOL[dtype], (kind, n, nrhs, err)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_sweep_scratch_reuse(slt, dtype):
    """Forward then backward on one scratch buffer (as potrs does), then a
    narrower right-hand side: each launch clears what it reads."""
    import torch
    n = 1500
    M = _triangle(n, True, 7, dtype)
    B = np.random.default_rng(3).uniform(-1, 1, (n, 8)).astype(dtype).astype(np.float64)
    Y, flags = _sweep(slt, torch, 2, M, B, dtype)
    X, flags = _sweep(slt, torch, 3, M, Y.astype(dtype).astype(np.float64), dtype, flags=flags)
    X1, _ = _sweep(slt, torch, 2, M, B[:, :2], dtype, flags=flags)
    Xr = _reference(3, M, _reference(2, M, B))
    assert np.abs(X - Xr).max() / np.abs(Xr).max() <= 4 * TOL[dtype]
    X1r = _reference(2, M, B[:, :2])
    assert np.abs(X1 - X1r).max() / np.abs(X1r).max() <= TOL[dtype]


@pytest.mark.parametrize("csize", ["1", "2", "4", "8"])
@pytest.mark.parametrize("kind", [2, 3, 0, 1])
@pytest.mark.parametrize("n,nrhs", [(4100, 16), (777, 9), (130, 8), (64, 5)])
def test_sweep16_cluster_sizes(slt, monkeypatch, csize, kind, n, nrhs):
    """The FP32 5-16 right-hand-side sweep for every cluster size
    (SLT_SWEEP_CLUSTER): consecutive blocks inside a cluster pass the chain
    input through distributed shared memory, across clusters through the
    mailbox; block counts that are not a multiple of the cluster size leave
    the last cluster's ranks partly idle."""
    import torch
    monkeypatch.setenv("SLT_SWEEP_CLUSTER", csize)
    uplo, _, _ = KINDS[kind]
    M = _triangle(n, uplo == "L", 31 * kind + n, np.float32)
    B = np.random.default_rng(n + kind).uniform(-1, 1, (n, nrhs)).astype(np.float32).astype(np.float64)
    X, _ = _sweep(slt, torch, kind, M, B, np.float32, ldm_pad=1 if n % 2 else 0)
    Xr = _reference(kind, M, B)
    err = np.abs(X - Xr).max() / np.abs(Xr).max()
    assert err <= TOL[np.float32], (csize, kind, n, nrhs, err)
