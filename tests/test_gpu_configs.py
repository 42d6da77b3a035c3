"""Parity at the solve configurations the benchmark reports, at their own sizes.

Each case runs the library's driver through the C ABI on the configuration's
matrix family and checks, independently of the library's kernels (cuBLAS
FP64 products on the device, or the host oracle):

* scaled backward error ||B - A X||_1 / (n ||A||_1 ||X||_1) (SLATE's tester,
  test/test_gesv.cc:330-380, test/test_posv.cc:300-345) <= 3 eps64 for the
  plain FP64 solves and <= 3 n eps64 for the mixed ones;
* forward error ||X - X_true||_max / ||X_true||_max <= kappa * 3 n eps64 where
  B = A X_true;
* refinement behaviour: iteration counts within one of the oracle's (the CPU
  restatement of SLATE's loops) on the same Philox inputs, at the largest
  sizes the oracle finishes in seconds (n = 8192 and 4096);
* the batched solver on systems up to n = 1024 (the panel-width-32 bucket),
  system by system against the oracle.

Sizes: config 2 is n = 16384 (4 RHS), config 3 n = 32768 (1 RHS,
kappa 1e2 and 1e4), config 4 n = 65536 (16 RHS, kappa 1e2).
"""
import numpy as np
import pytest

from gpu_util import EPS, berr, spd, to_dev, to_host

pytestmark = pytest.mark.gpu


def _berr_dev(torch, A, X, B):
    """Scaled backward error with cuBLAS FP64 (not the library's kernels)."""
    n = A.shape[0]
    R = B - A @ X
    return float(R.abs().sum(0).max() / (n * A.abs().sum(0).max() * X.abs().sum(0).max()))


def _ferr(torch, X, Xt):
    return float((X - Xt).abs().max() / Xt.abs().max())


def _ggt_dev(slt, torch, n, seed):
    """A = G G^T / n + I (G from SLATE's Philox normal stream; the product in
    FP32, as the benchmark forms it), made exactly symmetric in FP64."""
    G = slt.colmajor(torch.empty(n, n, dtype=torch.float64, device="cuda"))
    slt.generate(3, seed, G)
    Gf = G.to(torch.float32)
    del G
    torch.backends.cuda.matmul.allow_tf32 = False
    S = (Gf @ Gf.t()).to(torch.float64)
    del Gf
    S = torch.tril(S) + torch.tril(S, -1).t()
    S /= n
    S.diagonal().add_(1.0)
    return slt.colmajor(S)


def _sigma_dev(slt, torch, n, kappa, dist, spd_, seed=3):
    A = slt.colmajor(torch.empty(n, n, dtype=torch.float64, device="cuda"))
    slt.generate_sigma(A, kappa, dist, spd_, seed=seed)
    return A


def _xtrue(slt, torch, n, nrhs, seed=5):
    Xt = slt.colmajor(torch.empty(n, nrhs, dtype=torch.float64, device="cuda"))
    slt.generate(2, seed, Xt)
    return Xt


# ---------------------------------------------------------------------------
# config 2: posv n = 16384, nb = 512, 4 RHS, A = G G^T / n + I
@pytest.fixture(scope="module")
def config2_system(slt):
    import torch
    n, nrhs = 16384, 4
    A0 = _ggt_dev(slt, torch, n, 1)
    Xt = _xtrue(slt, torch, n, nrhs)
    B = slt.colmajor(A0 @ Xt)
    torch.cuda.synchronize()
    yield A0, Xt, B
    del A0, Xt, B
    torch.cuda.empty_cache()


@pytest.mark.parametrize("routine,prec", [("posv", "fp64"), ("posv_mixed", "fp16"), ("posv_mixed", "fp32")])
def test_config2_posv(slt, config2_system, routine, prec):
    import torch
    A0, Xt, B = config2_system
    n, nb, nrhs = A0.shape[0], 512, B.shape[1]
    kappa = 5.0                                  # ||A|| ||A^-1|| <= (1 + 4) / 1 for G G^T / n + I
    if routine == "posv":
        A = slt.colmajor(A0.clone())
        X = slt.colmajor(B.clone())
        info = slt.posv(A, X, slt.Options(nb=nb))
        bound = 3 * EPS
        del A
    else:
        X = slt.colmajor(torch.zeros(n, nrhs, dtype=torch.float64, device="cuda"))
        info, it, _ = slt.posv_mixed(A0, B, X, slt.Options(nb=nb, factor_precision=prec))
        assert it >= 0, it
        bound = 3 * n * EPS
    torch.cuda.synchronize()
    assert info == 0
    assert _berr_dev(torch, A0, X, B) <= bound
    assert _ferr(torch, X, Xt) <= kappa * 3 * n * EPS


# ---------------------------------------------------------------------------
# config 3: gesv_mixed n = 32768, nb = 512, 1 RHS, A = U diag(s) V^T, s geo
@pytest.mark.parametrize("kappa", [1e2, 1e4])
def test_config3_gesv_mixed(slt, kappa):
    import torch
    n, nb = 32768, 512
    A0 = _sigma_dev(slt, torch, n, kappa, "geo", False)
    Xt = _xtrue(slt, torch, n, 1)
    B = slt.colmajor(A0 @ Xt)
    A = slt.colmajor(A0.clone())
    for prec in ("fp32", "fp16"):
        X = slt.colmajor(torch.zeros(n, 1, dtype=torch.float64, device="cuda"))
        info, it, _ = slt.gesv_mixed(A, B, X, slt.Options(nb=nb, factor_precision=prec, refine="ir+gmres"))
        torch.cuda.synchronize()
        assert info == 0 and it >= 0, (prec, info, it)
        assert torch.equal(A, A0), prec          # A untouched: no FP64 fallback ran
        assert _berr_dev(torch, A0, X, B) <= 3 * n * EPS, prec
        assert _ferr(torch, X, Xt) <= kappa * 3 * n * EPS, prec
    del A, A0
    torch.cuda.empty_cache()


# ---------------------------------------------------------------------------
# config 4: posv_mixed_gmres n = 65536, nb = 512, 16 RHS, poev + logrand
def test_config4_posv_mixed_gmres(slt):
    import torch
    n, nb, nrhs, kappa = 65536, 512, 16, 1e2
    A = _sigma_dev(slt, torch, n, kappa, "logrand", True)
    Xt = _xtrue(slt, torch, n, nrhs)
    B = slt.colmajor(A @ Xt)
    X = slt.colmajor(torch.zeros(n, nrhs, dtype=torch.float64, device="cuda"))
    info, it, _ = slt.posv_mixed_gmres(A, B, X, slt.Options(nb=nb, factor_precision="fp16"))
    torch.cuda.synchronize()
    assert info == 0 and it >= 0, (info, it)
    assert slt.timer("posv_mixed_gmres::retry_fp32") < 0     # the FP16 factor sufficed
    assert _berr_dev(torch, A, X, B) <= 3 * n * EPS
    assert _ferr(torch, X, Xt) <= kappa * 3 * n * EPS
    del A, B, X
    torch.cuda.empty_cache()


# ---------------------------------------------------------------------------
# refinement behaviour against the oracle on the same inputs
def test_config2_family_iterations_match_oracle(orc, slt):
    """posv_mixed (SLATE's FP32 tier) at n = 8192, 4 RHS, G G^T / n + I."""
    import torch
    n, nb, nrhs = 8192, 512, 4
    A = spd(orc, n, 1)
    B = orc.generate(2, 2, n, nrhs)
    dA, dB = to_dev(A), to_dev(B)
    dX = to_dev(np.zeros((n, nrhs)))
    info, it, _ = slt.posv_mixed(dA, dB, dX, slt.Options(nb=nb))
    torch.cuda.synchronize()
    oinfo, oX, oit = orc.posv_mixed(A.copy(order="F"), B.copy(order="F"), nb)
    assert info == 0 and oinfo == 0
    assert it >= 0 and abs(it - oit) <= 1, (it, oit)
    assert berr(orc, A, to_host(dX), B, sym=True) <= 3 * n * EPS


def test_config4_family_iterations_match_oracle(orc, slt):
    """posv_mixed_gmres (FP32 tier) at n = 4096 with 16 RHS on the poev +
    logrand family: every column is SLATE's single-RHS FGMRES-IR; the worst
    column's count is compared."""
    import torch
    n, nb, nrhs = 4096, 512, 16
    A = orc.generate_sigma(n, 1e2, "logrand", True, 3)
    Xt = orc.generate(2, 5, n, nrhs)
    B = np.asfortranarray(A @ Xt)
    dA, dB = to_dev(A), to_dev(B)
    dX = to_dev(np.zeros((n, nrhs)))
    info, it, _ = slt.posv_mixed_gmres(dA, dB, dX, slt.Options(nb=nb))
    torch.cuda.synchronize()
    oinfo, oX, oit, ocol = orc.posv_mixed_gmres_nrhs(A.copy(order="F"), B, nb)
    assert info == 0 and oinfo == 0
    assert it >= 0 and abs(it - oit) <= 1, (it, oit, list(ocol))
    X = to_host(dX)
    assert berr(orc, A, X, B, sym=True) <= 3 * n * EPS
    assert np.abs(X - Xt).max() / np.abs(Xt).max() <= 1e2 * 3 * n * EPS


# ---------------------------------------------------------------------------
# config 5: batched systems up to n = 1024, system by system
def _batch(orc, sizes, seed):
    rng = np.random.default_rng(seed)
    out = []
    for t, n in enumerate(sizes):
        kind = t % 2
        A = spd(orc, n, 5000 + t) if kind == 1 else orc.generate(2, 6000 + t, n, n)
        r = int(rng.integers(1, 9))
        B = orc.generate(2, 7000 + t, n, r)
        out.append((kind, np.asfortranarray(A), np.asfortranarray(B)))
    return out


SIZES_LARGE = [513, 600, 700, 777, 800, 901, 1000, 1023, 1024, 1024, 520, 640, 960, 1020, 515, 1001]


def test_config5_batched_large_buckets_plain(orc, slt):
    import torch
    systems = _batch(orc, SIZES_LARGE, 11)
    dsys = [(k, slt.colmajor(to_dev(A)), slt.colmajor(to_dev(B))) for k, A, B in systems]
    vb = slt.VBatch(dsys)
    info = slt.solve_vbatched(vb)
    torch.cuda.synchronize()
    assert (info == 0).all()
    for t, ((k, A, B), (_, dA, dB)) in enumerate(zip(systems, dsys)):
        n = A.shape[0]
        X = to_host(dB)
        assert berr(orc, A, X, B, sym=(k == 1)) <= 3 * EPS, (t, n, k)
        if k == 0:
            oinfo, pt, po, oipiv, mg = orc.getrf(A.copy(order="F"), 32, 32, margins=True)
            gip = vb.ipiv_t[t][:n].cpu().numpy().astype(np.int64)
            robust = mg > 1 + 1e3 * n * EPS
            assert np.array_equal(gip[robust], oipiv[robust]), (t, n)


def test_config5_batched_large_buckets_mixed(orc, slt):
    import torch
    systems = _batch(orc, SIZES_LARGE, 12)
    dsys = [(k, slt.colmajor(to_dev(A)), slt.colmajor(to_dev(B))) for k, A, B in systems]
    Xs = [slt.colmajor(torch.zeros_like(dB)) for _, _, dB in dsys]
    vb = slt.VBatch(dsys, X=Xs)
    info, iters = slt.solve_mixed_vbatched(vb, slt.Options())
    torch.cuda.synchronize()
    assert (info == 0).all()
    assert (iters >= 0).all()
    for t, ((k, A, B), dX, (_, dA, _)) in enumerate(zip(systems, Xs, dsys)):
        n = A.shape[0]
        assert berr(orc, A, to_host(dX), B, sym=(k == 1)) <= 3 * n * EPS, (t, n, k)
        assert np.array_equal(to_host(dA), A)        # converged: A untouched
