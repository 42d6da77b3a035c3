"""The tensor-core FP64 residual (digit_residual.cu) against the exact residual.

slt_dresidual_digits forms R = B - A X from the digit planes of A (bytes,
rebuilt into BF16 digits in tensor memory) and the BF16 digits of X on the
tcgen05 tensor cores.  Checked here through the C ABI:

* accuracy against B - A X in extended precision (np.longdouble) on the
  host: |R - R_exact| <= 2^-50 n max_k|a_ik| max_k|x_kc| + 2^-51 (|b| +
  sum_k |a_ik||x_kc|) -- the bound of the dropped digits and classes plus
  the final roundings -- and no worse than 4x the FP64 kernel's own error
  (slt_dresidual) or 2^-52 of the row's magnitude sum;
* general and symmetric lower storage (the upper triangle holds NaN and
  must not be read), sizes off the 64 / 128 tile grid, leading dimensions
  above n, 1 to 16 right-hand sides, rows spread over 2^+-300, zero rows and
  columns, and a non-finite column of X (NaN in that column of R only);
* the mixed solvers with residual_engine 2 (tensor cores) against 1 (FP64):
  both converge to the tester's bound with iteration counts within one;
* ||A||_inf from the split's exact integer row sums
  (slt_dresidual_digits_norm), NaN for a non-finite entry.
"""
import ctypes

import numpy as np
import pytest

from gpu_util import EPS, berr, spd, to_dev, to_host

pytestmark = pytest.mark.gpu

i64, vp, cint = ctypes.c_int64, ctypes.c_void_p, ctypes.c_int


def _fns(slt):
    L = slt.lib()
    common = [i64, i64, vp, i64, cint, vp, i64, vp, i64, vp, i64]
    dg = L.slt_dresidual_digits
    dg.argtypes = common + [vp]
    dg.restype = cint
    fp = L.slt_dresidual
    fp.argtypes = common + [vp, vp]
    fp.restype = cint
    wsb = L.slt_residual_ws_bytes
    wsb.argtypes = [i64, i64]
    wsb.restype = ctypes.c_size_t
    return dg, fp, wsb


def _padded(M, ld):
    """Device column-major copy of M with leading dimension ld >= rows."""
    import torch
    m, n = M.shape
    P = np.full((ld, n), np.nan)
    P[:m] = M
    t = torch.from_numpy(np.ascontiguousarray(P.T)).cuda().t()
    return t


def _run(slt, A, X, B, sym, ld_pad=0):
    import torch
    dg, fp, wsb = _fns(slt)
    n, nrhs = X.shape
    lda, ldx, ldr = n + ld_pad, n + 2 * ld_pad, n + 3 * ld_pad
    dA, dX, dB = _padded(A, lda), _padded(X, ldx), _padded(B, ldx)
    dR = _padded(np.zeros((n, nrhs)), ldr)
    dF = _padded(np.zeros((n, nrhs)), ldr)
    s = vp(torch.cuda.current_stream().cuda_stream)
    rc = dg(n, nrhs, dA.data_ptr(), lda, sym, dB.data_ptr(), ldx, dX.data_ptr(), ldx, dR.data_ptr(), ldr, s)
    assert rc == 0, rc
    ws = torch.empty(wsb(n, nrhs), dtype=torch.uint8, device="cuda")
    rc = fp(n, nrhs, dA.data_ptr(), lda, sym, dB.data_ptr(), ldx, dX.data_ptr(), ldx, dF.data_ptr(), ldr,
            vp(ws.data_ptr()), s)
    assert rc == 0, rc
    torch.cuda.synchronize()
    return dR.cpu().numpy()[:n], dF.cpu().numpy()[:n]


def _check(A, X, B, R, F, sym):
    Af = np.tril(A) + np.tril(A, -1).T if sym else A
    n = A.shape[0]
    L = np.longdouble
    exact = (B.astype(L) - Af.astype(L) @ X.astype(L)).astype(np.float64)
    mag = np.abs(Af) @ np.abs(X)
    bound = (2.0 ** -50 * n * np.abs(Af).max(axis=1)[:, None] * np.abs(X).max(axis=0)[None, :]
             + 2.0 ** -51 * (np.abs(B) + mag))
    err = np.abs(R - exact)
    assert np.all(err <= bound), float(np.max(err / np.maximum(bound, 1e-300)))
    ferr = np.abs(F - exact)
    for c in range(X.shape[1]):
        lim = max(4 * ferr[:, c].max(), 2.0 ** -52 * mag[:, c].max())
        assert err[:, c].max() <= lim, (c, float(err[:, c].max()), float(ferr[:, c].max()))


@pytest.mark.parametrize("n,nrhs,sym,ld_pad", [
    (1000, 1, 0, 0), (1000, 16, 1, 0), (2100, 5, 0, 3), (2100, 16, 1, 5),
    (4096, 16, 0, 0), (777, 3, 1, 1), (130, 16, 0, 0), (64, 2, 1, 0)])
def test_digit_residual_accuracy(orc, slt, n, nrhs, sym, ld_pad):
    rng = np.random.default_rng(n + nrhs + sym)
    A = orc.generate(3, 11 + n, n, n)
    if sym:
        A = np.tril(A)
        A = A + np.tril(A, -1).T
    X = orc.generate(3, 12 + n, n, nrhs)
    B = A @ X + 1e-9 * orc.generate(2, 13 + n, n, nrhs)    # small residual: heavy cancellation
    Ain = A.copy()
    if sym:
        Ain[np.triu_indices(n, 1)] = np.nan       # never read in lower storage
    R, F = _run(slt, Ain, X, B, sym, ld_pad)
    _check(A, X, B, R, F, sym)


def test_digit_residual_scales_zeros_and_nonfinite(orc, slt):
    n, nrhs = 1500, 6
    rng = np.random.default_rng(3)
    A = orc.generate(3, 21, n, n) * np.ldexp(1.0, rng.integers(-300, 300, size=(n, 1)))
    A[17] = 0.0
    X = orc.generate(3, 22, n, nrhs) * np.ldexp(1.0, rng.integers(-30, 30, size=(1, nrhs)))
    X[:, 2] = 0.0
    X[::5, 4] *= 2.0 ** 40
    B = orc.generate(2, 23, n, nrhs)
    R, F = _run(slt, A, X, B, 0)
    _check(A, X, B, R, F, 0)
    assert np.array_equal(R[17], B[17])
    assert np.array_equal(R[:, 2], B[:, 2])
    X[100, 1] = np.inf
    R, _ = _run(slt, A, X, B, 0)
    assert np.all(np.isnan(R[:, 1]))
    others = [c for c in range(nrhs) if c != 1]
    assert np.all(np.isfinite(R[:, others]))


@pytest.mark.parametrize("chol", [1, 0])
def test_solvers_digit_vs_fp64_residual(orc, slt, chol):
    import torch
    n, nb, nrhs = 4096, 512, 16
    A = spd(orc, n, 31) if chol else orc.generate(2, 31, n, n)
    B = orc.generate(2, 32, n, nrhs)
    out = {}
    for eng in (1, 2):
        dA, dB = to_dev(A), to_dev(B)
        dX = to_dev(np.zeros((n, nrhs)))
        o = slt.Options(nb=nb, residual_engine=eng)
        f = slt.posv_mixed_gmres if chol else slt.gesv_mixed_gmres
        info, it, _ = f(dA, dB, dX, o)
        torch.cuda.synchronize()
        assert info == 0 and it >= 0, (eng, info, it)
        X = to_host(dX)
        assert berr(orc, A, X, B, sym=bool(chol)) <= 3 * n * EPS, eng
        out[eng] = it
        # IR (SLATE's gesv_mixed loop) with the same engine
        dX.zero_()
        f2 = slt.posv_mixed if chol else slt.gesv_mixed
        info, it2, _ = f2(to_dev(A), dB, dX, slt.Options(nb=nb, residual_engine=eng))
        torch.cuda.synchronize()
        assert info == 0 and it2 >= 0, (eng, info, it2)
        assert berr(orc, A, to_host(dX), B, sym=bool(chol)) <= 3 * n * EPS, eng
    assert abs(out[1] - out[2]) <= 1, out


@pytest.mark.parametrize("n,sym,ld_pad", [(1000, 0, 0), (2100, 1, 3), (4097, 1, 0), (777, 0, 1), (64, 1, 0)])
def test_digit_split_infinity_norm(slt, n, sym, ld_pad):
    """||A||_inf from the split's exact integer row sums of the fixed-point
    digits (slt_dresidual_digits_norm): rows spread over 2^+-300, a zero
    row, general and symmetric lower storage (the upper triangle holds NaN and
    must not be read); against the row sums of |A| in extended precision,
    within the rounding of the fixed-point digits; then a NaN entry makes the
    norm NaN."""
    import torch
    L = slt.lib()
    f = L.slt_dresidual_digits_norm
    f.argtypes = [i64, i64, vp, i64, cint, vp, i64, vp, i64, vp, i64, vp, vp]
    f.restype = cint
    rng = np.random.default_rng(n + sym)
    A = rng.standard_normal((n, n)) * np.ldexp(1.0, rng.integers(-300, 300, size=(n, 1)))
    if sym:
        A = np.tril(A) + np.tril(A, -1).T        # symmetric: row scales from both triangles
    A[n // 3, :] = 0.0
    A[:, n // 3] = 0.0
    Af = A.copy()
    if sym:
        A = np.where(np.tril(np.ones((n, n), dtype=bool)), A, np.nan)
    ref = float(np.max(np.abs(Af).astype(np.longdouble).sum(axis=1)))
    lda = n + ld_pad
    dA = _padded(A, lda)
    dN = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    s = vp(torch.cuda.current_stream().cuda_stream)
    assert f(n, 0, dA.data_ptr(), lda, sym, None, n, None, n, None, n, dN.data_ptr(), s) == 0
    torch.cuda.synchronize()
    got = float(dN.item())
    # every |a| enters as |F| 2^(e - 56), |F| = round(|a| 2^(56 - e)): at most
    # 2^(e - 57) off, and the row's largest entry is >= 2^(e - 2)
    assert abs(got - ref) <= (n * 2.0 ** -55 + 2.0 ** -50) * ref, (got, ref)
    # a NaN in the stored part
    A2 = A.copy()
    A2[n - 1, n // 2] = np.nan
    dA2 = _padded(A2, lda)
    assert f(n, 0, dA2.data_ptr(), lda, sym, None, n, None, n, None, n, dN.data_ptr(), s) == 0
    torch.cuda.synchronize()
    assert np.isnan(float(dN.item()))
