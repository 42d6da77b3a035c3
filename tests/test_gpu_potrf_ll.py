"""Left-looking tensor-core Cholesky of the mixed solvers (drivers.cc
potrf_ll_tc) and its two kernels.

* slt_tc_gemm_packed: C -= A B^T on operands already in FP16 / BF16 K-major
  rows, against torch's FP32 product of the same 16-bit values (relative
  1e-5 of the operands' magnitude sum), lower and full, sizes off the
  128-row tiles, leading dimensions above the rows;
* slt_pack_rows16: the row-major 16-bit copy of a block of the lower factor
  (exact rounding, zero above the diagonal, nothing written outside the
  block);
* the FP16 / BF16 mixed Cholesky solvers with the left-looking factor forced
  on (SLT_POTRF_LL=1), with and without the next block's update running
  beside the panels (SLT_LL_PANEL_SMS), against the right-looking one (=0):
  all converge to the tester's bound, iteration counts within one, and a
  non-SPD matrix ends in the FP64 fallback's info on every path (no wait
  runs out).
"""
import ctypes

import numpy as np
import pytest

from gpu_util import EPS, berr, spd, to_dev, to_host

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("tier", ["fp16", "bf16"])
@pytest.mark.parametrize("m,n,k,lower", [(300, 300, 128, 1), (1000, 257, 640, 1), (513, 130, 64, 0),
                                         (2048, 2048, 2048, 1)])
def test_tc_gemm_packed_matches_torch(slt, tier, m, n, k, lower):
    import torch
    L = slt.lib()
    f = L.slt_tc_gemm_packed
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
                  ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_void_p]
    dt = torch.float16 if tier == "fp16" else torch.bfloat16
    g = torch.Generator(device="cuda").manual_seed(m + n + k)
    lda16, ldb16 = k + 64, k + 128
    A = torch.zeros(m, lda16, dtype=dt, device="cuda")
    B = torch.zeros(n, ldb16, dtype=dt, device="cuda")
    A[:, :k] = torch.randn(m, k, generator=g, device="cuda").to(dt)
    B[:, :k] = torch.randn(n, k, generator=g, device="cuda").to(dt)
    A[:, k:] = float("nan")                       # beyond kpad: never read
    B[:, k:] = float("nan")
    ldc = ((m + 3) // 4) * 4 + 4
    C0 = torch.randn(n, ldc, generator=g, device="cuda", dtype=torch.float32)
    C = C0.clone()
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = f(slt._PREC_NAMES[tier], m, n, k, A.data_ptr(), lda16, B.data_ptr(), ldb16, C.data_ptr(), ldc, lower, s)
    assert rc == 0, rc
    torch.cuda.synchronize()
    P = A[:, :k].float() @ B[:, :k].float().t()   # m x n
    ref = C0[:, :m].t() - P                       # C is column-major: C[col, row]
    got = C[:, :m].t()
    scale = A[:, :k].float().abs() @ B[:, :k].float().abs().t() + 1.0
    if lower:
        mask = torch.tril(torch.ones(m, n, dtype=torch.bool, device="cuda"))
        assert torch.equal(got[~mask], C0[:, :m].t()[~mask])    # above the diagonal untouched
        ref = torch.where(mask, ref, got)
    assert ((got - ref).abs() <= 1e-5 * scale).all()
    assert torch.equal(C[:, m:], C0[:, m:])       # rows beyond m untouched


@pytest.mark.parametrize("tier", ["fp16", "bf16"])
def test_pack_rows16_layout(slt, tier):
    import torch
    L = slt.lib()
    f = L.slt_pack_rows16
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p,
                  ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]
    dt = torch.float16 if tier == "fp16" else torch.bfloat16
    n, lds, ldd = 777, 800, 832
    r0, c0, c1 = 300, 100, 357
    src = torch.randn(n, lds, device="cuda")       # column j at src[j, :] (column-major view)
    dst = torch.full((n, ldd), 7.0, dtype=dt, device="cuda")
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert f(slt._PREC_NAMES[tier], n, r0, c0, c1, src.data_ptr(), lds, dst.data_ptr(), ldd, s) == 0
    torch.cuda.synchronize()
    col = src[:, :n].t()                           # col[r, c] = element (r, c)
    blk = dst[r0:n, c0:c1].float()
    ref = col[r0:n, c0:c1].to(dt).float()
    rr = torch.arange(r0, n, device="cuda")[:, None]
    cc = torch.arange(c0, c1, device="cuda")[None, :]
    ref = torch.where(rr >= cc, ref, torch.zeros_like(ref))
    assert torch.equal(blk, ref)
    outside = torch.ones(n, ldd, dtype=torch.bool, device="cuda")
    outside[r0:n, c0:c1] = False
    assert (dst[outside].float() == 7.0).all()


@pytest.mark.parametrize("prec", ["fp16", "bf16"])
@pytest.mark.parametrize("n", [4096, 5000])
def test_mixed_cholesky_left_looking_vs_right_looking(orc, slt, monkeypatch, prec, n):
    import torch
    nrhs = 8
    A = spd(orc, n, 400 + n)
    B = orc.generate(2, 401 + n, n, nrhs)
    res = {}
    # left-looking without and with the next block's update beside the panels
    # (SLT_LL_PANEL_SMS: the panels' SM share), then right-looking
    for ll in ("1", "1:38", "0"):
        monkeypatch.setenv("SLT_POTRF_LL", ll[0])
        monkeypatch.setenv("SLT_LL_PANEL_SMS", ll[2:] if ":" in ll else "0")
        for name, fn in (("gmres", slt.posv_mixed_gmres), ("ir", slt.posv_mixed)):
            dX = to_dev(np.zeros((n, nrhs)))
            info, it, _ = fn(to_dev(A), to_dev(B), dX, slt.Options(nb=512, factor_precision=prec))
            torch.cuda.synchronize()
            assert info == 0 and it >= 0, (ll, name, info, it)
            assert berr(orc, A, to_host(dX), B, sym=True) <= 3 * n * EPS, (ll, name)
            res[(ll, name)] = it
    for name in ("gmres", "ir"):
        assert abs(res[("1", name)] - res[("0", name)]) <= 1, res
        assert abs(res[("1:38", name)] - res[("0", name)]) <= 1, res


def test_mixed_cholesky_left_looking_not_spd(orc, slt, monkeypatch):
    import torch
    n, bad = 4096, 2600
    A = spd(orc, n, 9)
    A[bad, bad] = -5.0
    B = orc.generate(2, 10, n, 2)
    for ll in ("1", "1:38", "0"):
        monkeypatch.setenv("SLT_POTRF_LL", ll[0])
        monkeypatch.setenv("SLT_LL_PANEL_SMS", ll[2:] if ":" in ll else "0")
        dX = to_dev(np.zeros((n, 2)))
        info, it, _ = slt.posv_mixed(to_dev(A), to_dev(B), dX, slt.Options(nb=512, factor_precision="fp16"))
        torch.cuda.synchronize()
        assert info == bad + 1 and it < 0, (ll, info, it)
