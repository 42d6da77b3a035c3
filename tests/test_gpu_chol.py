"""Cholesky parity on the GPU (potrf / potrs / posv) against the oracle."""
import numpy as np
import pytest

from gpu_util import EPS, berr, spd, to_dev, to_host

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,nb", [(1, 4), (5, 4), (64, 16), (100, 32), (300, 64), (1000, 256), (1300, 512),
                                  (45, 7), (77, 40), (530, 100)])
def test_potrf_parity(orc, slt, n, nb):
    import torch
    A = spd(orc, n, 40 + n)
    dA = to_dev(A)
    info = slt.potrf(dA, slt.Options(nb=nb))
    torch.cuda.synchronize()
    assert info == 0
    L = np.tril(to_host(dA))
    Ao = A.copy(order="F")
    assert orc.potrf(Ao, nb) == 0
    np.testing.assert_allclose(L, np.tril(Ao), atol=1e-12 * np.abs(Ao).max())
    # upper triangle untouched
    iu = np.triu_indices(n, 1)
    assert np.array_equal(to_host(dA)[iu], A[iu])


@pytest.mark.parametrize("n,nb,nrhs", [(200, 64, 1), (1024, 256, 4), (2048, 512, 16)])
def test_posv_backward_error(orc, slt, n, nb, nrhs):
    import torch
    A = spd(orc, n, 7)
    B = orc.generate(2, 8, n, nrhs)
    dA, dB = to_dev(A), to_dev(B)
    info = slt.posv(dA, dB, slt.Options(nb=nb))
    torch.cuda.synchronize()
    assert info == 0
    assert berr(orc, A, to_host(dB), B, sym=True) <= 3 * EPS


@pytest.mark.parametrize("bad", [0, 130, 150, 199])
def test_potrf_not_spd(orc, slt, bad):
    import torch
    n = 200
    A = spd(orc, n, 3)
    A[bad, bad] = -5.0
    dA = to_dev(A)
    info = slt.potrf(dA, slt.Options(nb=64))
    torch.cuda.synchronize()
    Ao = A.copy(order="F")
    assert info == orc.potrf(Ao, 64) == bad + 1


@pytest.mark.parametrize("bad", [600, 769, 1000, 1299])
def test_potrf_not_spd_wide_panel(orc, slt, bad):
    """A non-positive pivot in a later 64-column step of a 512-wide panel:
    found by the owner of that diagonal block while factoring it one step
    ahead; every block of the panel must stop at that step (info, no wait
    timing out)."""
    import torch
    n = 1300
    A = spd(orc, n, 3)
    A[bad, bad] = -5.0
    dA = to_dev(A)
    info = slt.potrf(dA, slt.Options(nb=512))
    torch.cuda.synchronize()
    assert info == orc.potrf(A.copy(order="F"), 512) == bad + 1


def test_potrf_known_answer_minij(orc, slt):
    import torch
    dA = to_dev(orc.generate_kind("minij", 70, 70))
    assert slt.potrf(dA, slt.Options(nb=32)) == 0
    torch.cuda.synchronize()
    np.testing.assert_allclose(np.tril(to_host(dA)), np.tril(np.ones((70, 70))), atol=1e-13)


@pytest.mark.parametrize("dtype", ["float64", "float32"])
@pytest.mark.parametrize("n", [12288, 20480])
def test_potrf_two_blocks_per_sm(slt, dtype, n):
    """n = 12288: the first panels need more 64-row blocks than SMs, so two
    panel blocks share an SM.  n = 20480: the first panels give every block
    two 64-row tiles (the general owner path and a multi-tile row solve).
    The factor must be run-to-run identical (no race between a block's own
    update and its next-step reads) and, in FP64, solve to backward error
    <= 3 eps and match torch's Cholesky; checked on the device with torch."""
    import torch
    tdt = getattr(torch, dtype)
    g = torch.Generator(device="cuda").manual_seed(11)
    G = torch.randn(n, n, device="cuda", dtype=torch.float64, generator=g)
    A = G @ G.t() / n + torch.eye(n, device="cuda", dtype=torch.float64)
    del G
    outs = []
    for _ in range(2):
        a = slt.colmajor(A.to(tdt))
        assert slt.potrf(a, slt.Options(nb=512)) == 0
        torch.cuda.synchronize()
        outs.append(torch.tril(a))
    assert torch.equal(outs[0], outs[1])
    if dtype == "float64":
        L = outs[0]
        b = torch.rand(n, 1, device="cuda", dtype=torch.float64, generator=g) * 2 - 1
        x = torch.cholesky_solve(b, L)
        r = b - A @ x
        berr = float(r.abs().max() / (A.abs().sum(1).max() * x.abs().max()))
        assert berr <= 3 * EPS, berr
        Lref = torch.linalg.cholesky(A)
        assert float((L - Lref).abs().max()) <= 1e-12 * float(A.abs().max())


@pytest.mark.parametrize("depth", [2, 4])
@pytest.mark.parametrize("n,nb", [(1300, 512), (530, 100), (2100, 256), (77, 40)])
def test_potrf_deferred_update_parity(orc, slt, monkeypatch, depth, n, nb):
    """Trailing update deferred over `depth` panels (each block column brought
    up to date with the block's earlier panels before it is factored): the
    same factor as the oracle's panel-by-panel potrf, the upper triangle
    untouched, and the first failing column reported on a non-SPD input."""
    import torch
    monkeypatch.setenv("SLT_LOOKAHEAD_PANEL_SMS", "0")
    monkeypatch.setenv("SLT_UPDATE_DEPTH", str(depth))
    A = spd(orc, n, 90 + n)
    dA = to_dev(A)
    assert slt.potrf(dA, slt.Options(nb=nb)) == 0
    torch.cuda.synchronize()
    Ao = A.copy(order="F")
    assert orc.potrf(Ao, nb) == 0
    np.testing.assert_allclose(np.tril(to_host(dA)), np.tril(Ao), atol=1e-12 * np.abs(Ao).max())
    iu = np.triu_indices(n, 1)
    assert np.array_equal(to_host(dA)[iu], A[iu])
    bad = min(n - 1, 3 * nb // 2 + 1)
    A[bad, bad] = -5.0
    dA = to_dev(A)
    info = slt.potrf(dA, slt.Options(nb=nb))
    torch.cuda.synchronize()
    assert info == orc.potrf(A.copy(order="F"), nb) == bad + 1


@pytest.mark.parametrize("depth", [2, 4])
def test_posv_mixed_fp16_deferred_update(orc, slt, monkeypatch, depth):
    import torch
    monkeypatch.setenv("SLT_LOOKAHEAD_PANEL_SMS", "0")
    monkeypatch.setenv("SLT_UPDATE_DEPTH", str(depth))
    n, nrhs = 4096, 4
    A = spd(orc, n, 5)
    B = orc.generate(2, 6, n, nrhs)
    dX = to_dev(np.zeros((n, nrhs)))
    info, it, _ = slt.posv_mixed_gmres(to_dev(A), to_dev(B), dX, slt.Options(nb=512, factor_precision="fp16"))
    torch.cuda.synchronize()
    assert info == 0 and it >= 0
    assert berr(orc, A, to_host(dX), B, sym=True) <= 3 * n * EPS
