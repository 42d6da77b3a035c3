"""Mixed-precision solvers on the GPU against the oracle.

Bar: converged (iter >= 0), FP64 backward error <= 3 n eps64, and the same
refinement behaviour as the oracle's restatement of SLATE's loop (iteration
counts within one).
"""
import numpy as np
import pytest

from gpu_util import EPS, berr, spd, to_dev, to_host

pytestmark = pytest.mark.gpu


def _run(slt, fn, A, B, opts):
    import torch
    dA, dB = to_dev(A), to_dev(B)
    dX = to_dev(np.zeros_like(B))
    info, it, _ = getattr(slt, fn)(dA, dB, dX, opts)
    torch.cuda.synchronize()
    return info, it, to_host(dX), to_host(dA)


@pytest.mark.parametrize("fn", ["gesv_mixed", "gesv_mixed_gmres", "posv_mixed", "posv_mixed_gmres"])
@pytest.mark.parametrize("n,nb", [(300, 64), (1500, 256)])
def test_mixed_parity(orc, slt, fn, n, nb):
    chol = fn.startswith("posv")
    A = spd(orc, n, 21) if chol else orc.generate(2, 22, n, n)
    nrhs = 1 if "gmres" in fn else 3
    B = orc.generate(2, 23, n, nrhs)
    info, it, X, Aout = _run(slt, fn, A, B, slt.Options(nb=nb))
    assert info == 0 and it >= 0
    assert berr(orc, A, X, B, sym=chol) <= 3 * n * EPS
    assert np.array_equal(Aout, A)          # A untouched unless the fallback runs
    Ao = A.copy(order="F")
    r = getattr(orc, fn)(Ao, B.copy(order="F") if nrhs > 1 else B[:, 0].copy(), nb)
    assert r[0] == 0 and abs(r[2] - it) <= 1


@pytest.mark.parametrize("fn", ["gesv_mixed", "posv_mixed_gmres"])
def test_mixed_forced_fallback(orc, slt, fn):
    chol = fn.startswith("posv")
    n = 400
    A = spd(orc, n, 31) if chol else orc.generate(2, 32, n, n)
    B = orc.generate(2, 33, n, 1)
    info, it, X, Aout = _run(slt, fn, A, B, slt.Options(nb=128, max_iterations=0))
    assert it == -1 and info == 0
    assert berr(orc, A, X, B, sym=chol) <= 3 * EPS


def test_mixed_singular(orc, slt):
    n = 256
    A = orc.generate(2, 3, n, n)
    A[:, 10] = 0.0
    B = orc.generate(2, 4, n, 1)
    info, it, X, _ = _run(slt, "gesv_mixed", A, B, slt.Options(nb=64, use_fallback=False))
    assert it == -3 and info == 11


@pytest.mark.parametrize("prec", ["tf32", "bf16", "fp16"])
@pytest.mark.parametrize("fn", ["gesv_mixed", "posv_mixed", "gesv_mixed_gmres"])
def test_tensor_core_tiers(orc, slt, fn, prec):
    """Low-precision tensor-core factorisations refined to FP64 accuracy."""
    chol = fn.startswith("posv")
    n, nb = 1536, 512
    A = spd(orc, n, 41) if chol else orc.generate(2, 42, n, n)
    nrhs = 1 if "gmres" in fn else 2
    B = orc.generate(2, 43, n, nrhs)
    info, it, X, Aout = _run(slt, fn, A, B, slt.Options(nb=nb, factor_precision=prec))
    assert info == 0
    if prec == "bf16" and not chol:
        # uniform random LU: kappa * u_bf16 > 1, refinement may stall; SLATE's
        # contract is then iter = -(itermax+1) and an FP64 fallback solution
        assert it >= 0 or it == -31
    else:
        assert it >= 0
    assert berr(orc, A, X, B, sym=chol) <= 3 * n * EPS
    if it >= 0:
        assert np.array_equal(Aout, A)


@pytest.mark.parametrize("fn", ["gesv_mixed", "gesv_mixed_gmres"])
def test_bf16_lu_converges_when_well_conditioned(orc, slt, fn):
    n, nb = 1024, 256
    A = orc.generate(2, 44, n, n) + np.eye(n) * (n / 8.0)
    A = np.asfortranarray(A)
    B = orc.generate(2, 45, n, 1)
    info, it, X, Aout = _run(slt, fn, A, B, slt.Options(nb=nb, factor_precision="bf16"))
    assert info == 0 and it >= 0
    assert berr(orc, A, X, B) <= 3 * n * EPS


def _butterfly_reference(n, cond, dist, spd, seed):
    """numpy restatement of the device generator (matgen.cu) for small n."""
    import oracle as O
    def unit_pair(i, level, key):
        a, b = O.philox(i, level, key)
        return (a >> 11) / float(1 << 53), b & 1
    if dist == "geo":
        s = cond ** (-np.arange(n) / (n - 1))
    else:
        s = np.array([np.exp(unit_pair(i, 0, seed)[0] * np.log(1.0 / cond)) for i in range(n)])
        s[0], s[1] = 1.0, 1.0 / cond
    A = np.diag(s)
    levels = int(np.ceil(np.log2(n)))
    for l in range(levels):
        h = 1 << l
        for side, key in (("rows", seed + 101), ("cols", seed + 101 if spd else seed + 202)):
            for blk in range(0, n, 2 * h):
                for i in range(blk, min(blk + h, n - h)):
                    k = i + h
                    u, bit = unit_pair(i, l, key)
                    th = 2 * np.pi * u
                    c, sn, si = np.cos(th), np.sin(th), (-1.0 if bit else 1.0)
                    if side == "rows":
                        x, y = si * A[i, :].copy(), A[k, :].copy()
                        A[i, :], A[k, :] = c * x + sn * y, -sn * x + c * y
                    else:
                        x, y = si * A[:, i].copy(), A[:, k].copy()
                        A[:, i], A[:, k] = c * x + sn * y, -sn * x + c * y
    return A, s


@pytest.mark.parametrize("dist,spd", [("geo", False), ("logrand", True)])
def test_generate_sigma_matches_restatement(orc, slt, dist, spd):
    import torch
    n, cond = 100, 1e4
    dA = slt.colmajor(torch.zeros(n, n, dtype=torch.float64, device="cuda"))
    slt.generate_sigma(dA, cond, dist, spd, seed=7)
    torch.cuda.synchronize()
    A = to_host(dA)
    R, s = _butterfly_reference(n, cond, dist, spd, 7)
    assert np.abs(A - R).max() <= 1e-12
    sv = np.linalg.svd(A, compute_uv=False)
    np.testing.assert_allclose(np.sort(sv), np.sort(s), rtol=1e-10)
    if spd:
        np.testing.assert_allclose(A, A.T, atol=1e-14)
        assert np.linalg.eigvalsh(A).min() > 0


@pytest.mark.parametrize("fn", ["gesv_mixed", "posv_mixed"])
def test_fp16_equilibration_of_badly_scaled_matrix(orc, slt, fn):
    """Rows and columns scaled by 2^-20 .. 2^20: the FP16 operands of the
    trailing update overflow without scaling; the power-of-two
    equilibration keeps them in range, and the FP64 refinement on the
    unscaled matrix still reaches FP64 backward error."""
    chol = fn.startswith("posv")
    n, nb = 1024, 256
    rng = np.random.default_rng(5)
    d = 2.0 ** rng.integers(-20, 21, n)
    if chol:
        A = np.asfortranarray(d[:, None] * spd(orc, n, 51) * d[None, :])
    else:
        e = 2.0 ** rng.integers(-20, 21, n)
        A = np.asfortranarray(d[:, None] * orc.generate(2, 52, n, n) * e[None, :])
    B = orc.generate(2, 53, n, 2)
    info, it, X, Aout = _run(slt, fn, A, B, slt.Options(nb=nb, factor_precision="fp16", equilibrate=1))
    assert info == 0 and it >= 0
    assert berr(orc, A, X, B, sym=chol) <= 3 * n * EPS
    assert np.array_equal(Aout, A)


def _sigma_system(slt, n, cond, seed, spd):
    import torch
    dA = slt.colmajor(torch.zeros(n, n, dtype=torch.float64, device="cuda"))
    slt.generate_sigma(dA, cond, "logrand" if spd else "geo", spd, seed=seed)
    torch.cuda.synchronize()
    return to_host(dA)


@pytest.mark.parametrize("kappa", [1e4, 1e6])
@pytest.mark.parametrize("fn", ["gesv_mixed", "posv_mixed"])
def test_ill_conditioned_16bit_without_fp64_fallback(orc, slt, fn, kappa):
    """FP16 factors at kappa = 1e4, 1e6: plain IR contracts by about
    kappa * u_fp16 per step and may diverge.  The ir+gmres chain continues
    stalled columns with FGMRES-IR on the same factors; if that fails too,
    the FP32 retry refactors in FP32 -- in every case the answer reaches FP64
    backward error without SLATE's FP64 fallback (A left untouched)."""
    chol = fn.startswith("posv")
    n, nb = 2048, 256
    A = _sigma_system(slt, n, kappa, 61, chol)
    xt = orc.generate(2, 62, n, 1)
    B = np.asfortranarray(A @ xt)
    _, it_ir, _, _ = _run(slt, fn, A, B, slt.Options(nb=nb, factor_precision="fp16", lo_retry=0))
    _, it_ch, _, _ = _run(slt, fn, A, B, slt.Options(nb=nb, factor_precision="fp16", refine="ir+gmres",
                                                     lo_retry=0))
    info, it, X, Aout = _run(slt, fn, A, B, slt.Options(nb=nb, factor_precision="fp16", refine="ir+gmres"))
    retried = slt.timer(fn + "::retry_fp32") > 0
    print(fn, kappa, "ir:", it_ir, "ir+gmres:", it_ch, "with fp32 retry:", it, retried)
    assert info == 0 and it >= 0
    assert np.array_equal(Aout, A)          # no FP64 fallback
    assert retried == (it_ch < 0)
    assert berr(orc, A, X, B, sym=chol) <= 3 * n * EPS
    assert np.abs(X - xt).max() / np.abs(xt).max() <= kappa * 3 * n * EPS


def _spd_kappa(n, kappa, seed):
    """Q diag(s) Q^T, s geometric from 1 to 1/kappa (Haar Q from a seed)."""
    rng = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    return np.asfortranarray((Q * np.geomspace(1.0, 1.0 / kappa, n)) @ Q.T)


@pytest.mark.parametrize("fn", ["posv_mixed", "posv_mixed_gmres"])
def test_fp8_tier_converges_when_kappa_small(orc, slt, fn):
    """FP8 E4M3 trailing updates (per-tile power-of-two scales): kappa = 10
    converges in a handful of steps to the FP64 bar."""
    n = 1024
    A = _spd_kappa(n, 10.0, 31)
    B = orc.generate(2, 32, n, 2)
    info, it, X, Aout = _run(slt, fn, A, B, slt.Options(nb=256, factor_precision="fp8", lo_retry=0))
    assert info == 0 and 0 <= it <= 12, it
    assert berr(orc, A, X, B, sym=True) <= 3 * n * EPS
    assert np.array_equal(Aout, A)


def test_fp8_tier_falls_back_when_kappa_large(orc, slt):
    """kappa = 1e4 is beyond E4M3's 3-bit mantissa: no convergence in itermax
    steps, iter = -(itermax + 1) and the FP64 fallback's solution; with the
    ladder on, the FP32 retry converges instead."""
    n = 768
    A = _spd_kappa(n, 1e4, 33)
    B = orc.generate(2, 34, n, 1)
    info, it, X, _ = _run(slt, "posv_mixed", A, B, slt.Options(nb=256, factor_precision="fp8", lo_retry=0,
                                                                   max_iterations=10))
    assert info == 0 and it == -11
    assert berr(orc, A, X, B, sym=True) <= 3 * EPS
    info, it, X, Aout = _run(slt, "posv_mixed", A, B, slt.Options(nb=256, factor_precision="fp8"))
    assert info == 0 and it >= 0
    assert berr(orc, A, X, B, sym=True) <= 3 * n * EPS
    assert np.array_equal(Aout, A)


def test_fp8_tier_lu(orc, slt):
    """The LU form: a diagonally dominant general matrix converges with FP8
    updates."""
    n = 1024
    A = np.asfortranarray(orc.generate(2, 35, n, n) + 0.25 * n * np.eye(n))
    B = orc.generate(2, 36, n, 2)
    info, it, X, _ = _run(slt, "gesv_mixed", A, B, slt.Options(nb=256, factor_precision="fp8", lo_retry=0))
    assert info == 0 and it >= 0
    assert berr(orc, A, X, B) <= 3 * n * EPS


@pytest.mark.parametrize("fn", ["gesv_mixed", "posv_mixed"])
def test_tf32x3_tier_matches_fp32(orc, slt, fn):
    """The split-precision 3xTF32 tier refines like the FP32 tier (iteration
    count within one) to the same FP64 bar."""
    n = 1500
    chol = fn.startswith("posv")
    A = spd(orc, n, 41) if chol else orc.generate(2, 42, n, n)
    B = orc.generate(2, 43, n, 2)
    info, it, X, _ = _run(slt, fn, A, B, slt.Options(nb=256, factor_precision="tf32x3"))
    info32, it32, _, _ = _run(slt, fn, A, B, slt.Options(nb=256, factor_precision="fp32"))
    assert info == 0 and it >= 0 and abs(it - it32) <= 1, (it, it32)
    assert berr(orc, A, X, B, sym=chol) <= 3 * n * EPS
