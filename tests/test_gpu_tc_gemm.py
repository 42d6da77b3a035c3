"""tcgen05 low-precision trailing update against a plain PyTorch fp32 reference.

C (fp32) -= round(A) op(round(B)) where round() is the tier's operand type
(BF16, FP16, or TF32 with round-to-nearest-away).  The reference multiplies
the same rounded operands in fp32 (TF32 math off); differences come only from
the fp32 accumulation order: |err| <= 1e-5 * k * max|A| max|B| is asserted.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TIERS = {"tf32": 2, "bf16": 3, "fp16": 4, "fp8": 5, "tf32x3": 6}


def _round(torch, x, tier):
    if tier == "bf16":
        return x.to(torch.bfloat16).float()
    if tier == "fp16":
        return x.to(torch.float16).float()
    i = x.contiguous().view(torch.int32)
    r = ((i + 0x1000) & ~0x1FFF)
    return r.view(torch.float32)


def _call(slt, tier, transb, A, B, C, lower):
    import torch
    L = slt.lib()
    f = L.slt_tc_gemm_update
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_char, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p,
                  ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int,
                  ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
    m, n = C.shape
    k = A.shape[1]
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = f(TIERS[tier], transb.encode(), m, n, k, A.data_ptr(), A.stride(1), B.data_ptr(), B.stride(1),
           C.data_ptr(), C.stride(1), int(lower), None, 0, s)
    assert rc == 0, rc
    torch.cuda.synchronize()
    L.slt_tc_status.restype = ctypes.c_int
    assert L.slt_tc_status() == 0


@pytest.mark.parametrize("tier", ["bf16", "fp16", "tf32"])
@pytest.mark.parametrize("m,n,k,transb", [(128, 128, 64, "N"), (300, 200, 100, "N"), (129, 257, 33, "N"),
                                          (1024, 768, 512, "N"), (640, 384, 256, "T"), (77, 500, 512, "T"),
                                          (40000, 200, 64, "N"), (20000, 328, 128, "T")])
def test_tc_update_matches_torch(slt, tier, m, n, k, transb):
    import torch
    torch.backends.cuda.matmul.allow_tf32 = False
    g = torch.Generator(device="cuda").manual_seed(m * 7 + n + k)
    A = slt.colmajor(torch.randn(m, k, device="cuda", generator=g))
    B = slt.colmajor(torch.randn(k, n, device="cuda", generator=g) if transb == "N"
                     else torch.randn(n, k, device="cuda", generator=g))
    C0 = torch.randn(m, n, device="cuda", generator=g)
    C = slt.colmajor(C0.clone())
    opB = _round(torch, B, tier) if transb == "N" else _round(torch, B, tier).t()
    ref = C0 - _round(torch, A, tier) @ opB
    _call(slt, tier, transb, A, B, C, 0)
    tol = 1e-5 * k * float(A.abs().max() * B.abs().max())
    err = float((C - ref).abs().max())
    assert err <= tol, (err, tol)


@pytest.mark.parametrize("tier", ["bf16", "tf32"])
def test_tc_update_lower(slt, tier):
    import torch
    torch.backends.cuda.matmul.allow_tf32 = False
    n, k = 700, 192
    g = torch.Generator(device="cuda").manual_seed(5)
    L = slt.colmajor(torch.randn(n, k, device="cuda", generator=g))
    C0 = torch.randn(n, n, device="cuda", generator=g)
    C = slt.colmajor(C0.clone())
    Lr = _round(torch, L, tier)
    ref = C0 - Lr @ Lr.t()
    _call(slt, tier, "T", L, L, C, 1)
    low = torch.tril(torch.ones(n, n, device="cuda", dtype=torch.bool))
    tol = 1e-5 * k * float(L.abs().max() ** 2)
    assert float((C - ref)[low].abs().max()) <= tol
    assert torch.equal(C[~low], C0[~low])


def _fp8_tiles(torch, X):
    """X (rows x k) with each 128-row tile scaled by 2^(8 - e), max|tile| =
    m 2^e, rounded to E4M3 and scaled back: the FP8 tier's operand."""
    out = torch.empty_like(X)
    for t in range(0, X.shape[0], 128):
        blk = X[t:t + 128]
        mx = blk.abs().max()
        s = 1.0
        if float(mx) > 0:
            _, e = torch.frexp(mx)
            s = 2.0 ** (8 - int(e))
        out[t:t + 128] = (blk * s).to(torch.float8_e4m3fn).float() / s
    return out


@pytest.mark.parametrize("m,n,k,transb", [(128, 128, 64, "N"), (300, 200, 100, "N"), (129, 257, 33, "N"),
                                          (1024, 768, 512, "N"), (640, 384, 256, "T"), (77, 500, 512, "T"),
                                          (20000, 328, 128, "T")])
def test_tc_update_fp8(slt, m, n, k, transb):
    """FP8 E4M3 tier: per-128-row-tile power-of-two scales, FP32 accumulation."""
    import torch
    torch.backends.cuda.matmul.allow_tf32 = False
    g = torch.Generator(device="cuda").manual_seed(m * 3 + n + k)
    A = slt.colmajor(torch.randn(m, k, device="cuda", generator=g) * 7.0)
    B = slt.colmajor(torch.randn(k, n, device="cuda", generator=g) * 0.01 if transb == "N"
                     else torch.randn(n, k, device="cuda", generator=g) * 0.01)
    C0 = torch.randn(m, n, device="cuda", generator=g)
    C = slt.colmajor(C0.clone())
    Bt = B.t() if transb == "N" else B              # n x k, the operand's rows
    A8, B8 = _fp8_tiles(torch, A.contiguous()), _fp8_tiles(torch, Bt.contiguous())
    ref = C0 - A8 @ B8.t()
    _call(slt, "fp8", transb, A, B, C, 0)
    tol = 1e-5 * k * float(A8.abs().max() * B8.abs().max())
    err = float((C - ref).abs().max())
    assert err <= tol, (err, tol)
    # the quantisation error itself is that of a 3-bit mantissa: far above the tol
    assert float((ref - (C0 - A @ Bt.t())).abs().max()) > 10 * tol


def test_tc_update_fp8_lower(slt):
    import torch
    n, k = 700, 192
    g = torch.Generator(device="cuda").manual_seed(9)
    L = slt.colmajor(torch.randn(n, k, device="cuda", generator=g))
    C0 = torch.randn(n, n, device="cuda", generator=g)
    C = slt.colmajor(C0.clone())
    L8 = _fp8_tiles(torch, L.contiguous())
    ref = C0 - L8 @ L8.t()
    _call(slt, "fp8", "T", L, L, C, 1)
    low = torch.tril(torch.ones(n, n, device="cuda", dtype=torch.bool))
    tol = 1e-5 * k * float(L8.abs().max()) ** 2
    assert float((C - ref)[low].abs().max()) <= tol
    assert torch.equal(C[~low], C0[~low])


@pytest.mark.parametrize("m,n,k,transb", [(128, 128, 64, "N"), (300, 200, 100, "N"), (1024, 768, 512, "N"),
                                          (640, 384, 256, "T"), (77, 500, 512, "T"), (20000, 328, 128, "T")])
def test_tc_update_tf32x3(slt, m, n, k, transb):
    """Split-precision 3xTF32: C -= A op(B) to near-FP32 accuracy on the
    tensor cores; compared with an FP64 product, the error stays at the
    scale of FP32 rounding (far below a single TF32 product's)."""
    import torch
    g = torch.Generator(device="cuda").manual_seed(m + 5 * n + k)
    A = slt.colmajor(torch.randn(m, k, device="cuda", generator=g))
    B = slt.colmajor(torch.randn(k, n, device="cuda", generator=g) if transb == "N"
                     else torch.randn(n, k, device="cuda", generator=g))
    C0 = torch.randn(m, n, device="cuda", generator=g)
    C = slt.colmajor(C0.clone())
    opB = B if transb == "N" else B.t()
    ref = C0.double() - A.double() @ opB.double()
    _call(slt, "tf32x3", transb, A, B, C, 0)
    scale = float((A.abs().double() @ opB.abs().double()).max()) + float(C0.abs().max())
    err = float((C.double() - ref).abs().max())
    assert err <= 2e-6 * scale, (err, scale)
    # a single TF32 product is ~100x further off
    Ct = slt.colmajor(C0.clone())
    _call(slt, "tf32", transb, A, B, Ct, 0)
    assert float((Ct.double() - ref).abs().max()) > 10 * err
