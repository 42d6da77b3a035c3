"""Random butterfly transforms and gesv_rbt on the GPU against the oracle's
restatement of SLATE's gerbt / gesv_rbt.

Bar: the butterfly kernels reproduce the oracle bit for bit on the same
diagonals (both round every product and sum once, in Tile_gerbt.hh's order);
the random diagonal matches exp(r / 20) of the Philox stream to 2 ulp (CUDA's
exp and numpy's may differ in the last bit); gesv_rbt reaches backward error
<= 3 eps64 with the oracle's iteration count +- 1 on the same diagonals, and
falls back to partial pivoting (iter = -(itermax + 1)) when refinement fails.
"""
import numpy as np
import pytest

from gpu_util import EPS, to_dev, to_host

pytestmark = pytest.mark.gpu


def _diag(rng, n):
    return np.exp(rng.uniform(-1, 1, n) / 20.0)


def _vec(x):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


@pytest.mark.parametrize("n,nb,d", [(300, 64, 2), (257, 32, 3), (1000, 96, 2), (64, 64, 1), (5, 8, 2), (130, 32, 0)])
def test_gerbt_bit_exact(orc, slt, n, nb, d):
    import torch
    rng = np.random.default_rng(n + nb + d)
    A = np.asfortranarray(rng.uniform(-1, 1, (n, n)))
    B = np.asfortranarray(rng.uniform(-1, 1, (n, 3)))
    u, v = _diag(rng, n), _diag(rng, n)
    dA, dB = to_dev(A), to_dev(B)
    slt.gerbt2(dA, _vec(u), _vec(v), d, nb)
    torch.cuda.synchronize()
    assert np.array_equal(to_host(dA), orc.gerbt2(A, u, v, d, nb))
    for trans in ("T", "N"):
        dB = to_dev(B)
        slt.gerbt1(trans, dB, _vec(u), d, nb)
        torch.cuda.synchronize()
        assert np.array_equal(to_host(dB), orc.gerbt1(trans, B, u, d, nb)), trans


def test_rbt_diag(orc, slt):
    n = 777
    w = slt.rbt_diag(n, 42).cpu().numpy()
    r = orc.generate(2, 42, n, 1)[:, 0]
    np.testing.assert_allclose(w, np.exp(r / 20.0), rtol=4 * EPS, atol=0)
    assert (w > np.exp(-0.05) * (1 - 1e-15)).all() and (w < np.exp(0.05) * (1 + 1e-15)).all()


def _berr(A, X, B):
    return np.abs(B - A @ X).sum(0).max() / (A.shape[0] * np.abs(A).sum(0).max() * np.abs(X).sum(0).max())


@pytest.mark.parametrize("n,nb,nrhs", [(500, 128, 3), (333, 64, 1)])
def test_gesv_rbt_matches_oracle(orc, slt, n, nb, nrhs):
    import torch
    A = orc.generate(2, 401, n, n)
    B = orc.generate(2, 402, n, nrhs)
    dA, dB = to_dev(A), to_dev(B)
    dX = to_dev(np.zeros((n, nrhs)))
    info, it = slt.gesv_rbt(dA, dB, dX, slt.Options(nb=nb, ib=16))
    torch.cuda.synchronize()
    assert info == 0 and it >= 0
    X = to_host(dX)
    assert _berr(A, X, B) <= 3 * EPS
    mt = -(-n // nb)
    u = slt.rbt_diag(n, 42).cpu().numpy()
    v = slt.rbt_diag(n, 42 + mt).cpu().numpy()
    Xo, ito, infoo = orc.gesv_rbt(A, B, nb, u, v, depth=2, ib=16)
    assert infoo == 0 and abs(ito - it) <= 1, (it, ito)
    np.testing.assert_allclose(X, Xo, rtol=0, atol=1e-9 * np.abs(Xo).max())
    # B untouched; A holds the no-pivoting factors of W_U^T A W_V
    assert np.array_equal(to_host(dB), B)
    Ap = orc.gerbt2(A, u, v, 2, nb)
    LU = to_host(dA)
    L = np.tril(LU, -1) + np.eye(n)
    U = np.triu(LU)
    assert np.abs(L @ U - Ap).max() <= 1e3 * n * EPS * np.abs(Ap).max()


def test_gesv_rbt_zero_leading_pivot(orc, slt):
    """a11 = 0: LU without pivoting of A itself stops at column 1; after the
    transform it runs through."""
    import torch
    n = 256
    A = orc.generate(2, 403, n, n)
    A[0, 0] = 0.0
    B = orc.generate(2, 404, n, 2)
    dA = to_dev(A)
    info_np, _ = slt.getrf(dA, slt.Options(nb=64, pivot_threshold=0.0))
    torch.cuda.synchronize()
    assert info_np == 1
    dA, dB, dX = to_dev(A), to_dev(B), to_dev(np.zeros((n, 2)))
    info, it = slt.gesv_rbt(dA, dB, dX, slt.Options(nb=64))
    torch.cuda.synchronize()
    assert info == 0 and 0 <= it <= 5
    assert _berr(A, to_host(dX), B) <= 3 * EPS


def test_gesv_rbt_fallback(orc, slt):
    """A stopping test no residual can meet and one refinement step: not
    converged -> iter = -2 and the partial-pivoting solve; A is left as it
    was (SLATE restores it before the fallback)."""
    import torch
    n = 200
    A = orc.generate(2, 410, n, n)
    B = orc.generate(2, 405, n, 1)
    dA, dB, dX = to_dev(A), to_dev(B), to_dev(np.zeros((n, 1)))
    info, it = slt.gesv_rbt(dA, dB, dX, slt.Options(nb=64, max_iterations=1, tolerance=1e-300))
    torch.cuda.synchronize()
    assert it == -2 and info == 0
    assert np.array_equal(to_host(dA), A)
    assert _berr(A, to_host(dX), B) <= 3 * EPS
    Xo, ito, _ = orc.gesv_rbt(A, B, 64, np.ones(n), np.ones(n), itermax=1, tol=1e-300)
    assert ito == -2


def test_gesv_rbt_no_refinement(orc, slt):
    import torch
    n = 300
    A = orc.generate(2, 406, n, n)
    B = orc.generate(2, 407, n, 2)
    dA, dB, dX = to_dev(A), to_dev(B), to_dev(np.zeros((n, 2)))
    info, it = slt.gesv_rbt(dA, dB, dX, slt.Options(nb=64, max_iterations=0))
    torch.cuda.synchronize()
    assert info == 0 and it == 0
    assert _berr(A, to_host(dX), B) <= 1e3 * EPS


def test_gesv_rbt_singular_reports_info(orc, slt):
    import torch
    n = 120
    A = orc.generate(2, 408, n, n)
    A[:, 17] = 0.0
    B = orc.generate(2, 409, n, 1)
    dA, dB, dX = to_dev(A), to_dev(B), to_dev(np.zeros((n, 1)))
    info, it = slt.gesv_rbt(dA, dB, dX, slt.Options(nb=32, max_iterations=3))
    torch.cuda.synchronize()
    assert it == -4
    Ao, Bo = A.copy(order="F"), B.copy(order="F")
    oinfo, _, _ = orc.gesv(Ao, Bo, 32)
    assert info == oinfo > 0
