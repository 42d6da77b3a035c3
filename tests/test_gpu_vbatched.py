"""Variable-size batched solves on the GPU against the oracle, per system,
for sizes from 1 to 1024 (config 5's range, across the tuning table's
switch of panel width).

Bar: every system's pivots equal the oracle's (SLATE's getrf restated) on
rows whose pivot margin exceeds rounding; FP64 backward error <= 3 eps64
(plain) or 3 n eps64 (mixed); SLATE's info on singular / indefinite systems;
A and B untouched by a converged mixed solve.
"""
import numpy as np
import pytest

from gpu_util import EPS, berr, spd, to_dev, to_host

pytestmark = pytest.mark.gpu


def _systems(orc, sizes, seed, nrhs_max=8, kinds=None):
    rng = np.random.default_rng(seed)
    out = []
    for t, n in enumerate(sizes):
        kind = int(kinds[t]) if kinds is not None else int(rng.integers(0, 2))
        A = spd(orc, n, 1000 + t) if (kind == 1 and n > 0) else (
            orc.generate(2, 2000 + t, n, n) if n > 0 else np.zeros((0, 0), order="F"))
        r = int(rng.integers(1, nrhs_max + 1))
        B = orc.generate(2, 3000 + t, n, r) if n > 0 else np.zeros((0, r), order="F")
        out.append((kind, np.asfortranarray(A), np.asfortranarray(B)))
    return out


def _to_dev_systems(slt, systems):
    import torch
    dev = []
    for k, A, B in systems:
        dA = to_dev(A) if A.size else torch.zeros(0, 0, dtype=torch.float64, device="cuda")
        dB = to_dev(B) if B.size else torch.zeros(0, B.shape[1], dtype=torch.float64, device="cuda")
        dev.append((k, slt.colmajor(dA), slt.colmajor(dB)))
    return dev


SIZES = [1, 2, 3, 5, 17, 31, 32, 33, 47, 63, 64, 65, 96, 127, 128, 129, 200, 257, 300, 0]


def test_vbatched_plain_matches_oracle(orc, slt):
    import torch
    systems = _systems(orc, SIZES, 1, nrhs_max=11)
    dsys = _to_dev_systems(slt, systems)
    vb = slt.VBatch(dsys)
    info = slt.solve_vbatched(vb)
    torch.cuda.synchronize()
    assert (info == 0).all()
    for t, ((k, A, B), (_, dA, dB)) in enumerate(zip(systems, dsys)):
        n = A.shape[0]
        if n == 0:
            continue
        X = to_host(dB)
        assert berr(orc, A, X, B, sym=(k == 1)) <= 3 * EPS, (t, n, k)
        if k == 0:
            oinfo, pt, po, oipiv, mg = orc.getrf(A.copy(order="F"), 32, 32, margins=True)
            gip = vb.ipiv_t[t][:n].cpu().numpy().astype(np.int64)
            robust = mg > 1 + 1e3 * n * EPS
            assert np.array_equal(gip[robust], oipiv[robust]), (t, n)
        else:
            L = np.tril(to_host(dA))
            np.testing.assert_allclose(L, np.linalg.cholesky(A), rtol=0, atol=1e-12 * np.abs(A).max())


def test_vbatched_plain_info(orc, slt):
    import torch
    n = 70
    A1 = orc.generate(2, 5, n, n)
    A1[:, 40] = 0.0                       # exact zero pivot at column 41
    A2 = spd(orc, n, 6)
    A2[50, 50] = -1.0                     # leading minor 51 not positive
    B = orc.generate(2, 7, n, 2)
    systems = [(0, np.asfortranarray(A1), B.copy(order="F")), (1, np.asfortranarray(A2), B.copy(order="F")),
               (0, orc.generate(2, 8, n, n), B.copy(order="F"))]
    dsys = _to_dev_systems(slt, systems)
    info = slt.solve_vbatched(slt.VBatch(dsys))
    torch.cuda.synchronize()
    assert info[0] == 41
    assert info[1] == orc.potrf(np.asfortranarray(A2.copy()), 32) == 51
    assert info[2] == 0


def test_vbatched_mixed_converges(orc, slt):
    import torch
    systems = _systems(orc, SIZES, 2)
    dsys = _to_dev_systems(slt, systems)
    X = [slt.colmajor(torch.zeros_like(b)) for _, _, b in dsys]
    vb = slt.VBatch(dsys, X=X)
    info, it = slt.solve_mixed_vbatched(vb, slt.Options())
    torch.cuda.synchronize()
    assert (info == 0).all() and (it >= 0).all(), it
    for t, ((k, A, B), (_, dA, dB), x) in enumerate(zip(systems, dsys, X)):
        n = A.shape[0]
        if n == 0:
            continue
        assert berr(orc, A, to_host(x), B, sym=(k == 1)) <= 3 * n * EPS, (t, n, k)
        assert np.array_equal(to_host(dA), A) and np.array_equal(to_host(dB), B)
        # iteration count within one of the oracle's gesv_mixed / posv_mixed (one tile: nb = n)
        Ao = A.copy(order="F")
        r = (orc.posv_mixed(Ao, B.copy(order="F"), max(n, 1)) if k == 1
             else orc.gesv_mixed(Ao, B.copy(order="F"), max(n, 1)))
        assert r[0] == 0 and abs(r[2] - it[t]) <= 1, (t, n, r[2], it[t])


def test_vbatched_mixed_forced_fallback(orc, slt):
    import torch
    systems = _systems(orc, [40, 130, 7], 3)
    dsys = _to_dev_systems(slt, systems)
    X = [slt.colmajor(torch.zeros_like(b)) for _, _, b in dsys]
    vb = slt.VBatch(dsys, X=X)
    info, it = slt.solve_mixed_vbatched(vb, slt.Options(max_iterations=0))
    torch.cuda.synchronize()
    assert (it == -1).all() and (info == 0).all()
    for (k, A, B), x in zip(systems, X):
        assert berr(orc, A, to_host(x), B, sym=(k == 1)) <= 3 * EPS


def test_vbatched_rejects_oversize(slt):
    import torch
    a = slt.colmajor(torch.zeros(2049, 2049, dtype=torch.float64, device="cuda"))
    b = slt.colmajor(torch.zeros(2049, 1, dtype=torch.float64, device="cuda"))
    with pytest.raises(slt.SlateError):
        slt.solve_vbatched(slt.VBatch([(0, a, b)]))


@pytest.mark.parametrize("pb", [16, 32])
def test_vbatched_plain_panel_width(orc, slt, monkeypatch, pb):
    """Both panel widths the tuning table can pick: same backward error bar,
    and the pivots of either width equal the oracle's (partial pivoting does
    not depend on the blocking) on rows with a clear pivot margin."""
    import torch
    monkeypatch.setenv("SLT_VBATCHED_PB", str(pb))
    systems = _systems(orc, [15, 16, 17, 33, 100, 161, 250], 7, nrhs_max=9)
    dsys = _to_dev_systems(slt, systems)
    vb = slt.VBatch(dsys)
    info = slt.solve_vbatched(vb)
    torch.cuda.synchronize()
    assert (info == 0).all()
    for t, ((k, A, B), (_, dA, dB)) in enumerate(zip(systems, dsys)):
        n = A.shape[0]
        assert berr(orc, A, to_host(dB), B, sym=(k == 1)) <= 3 * EPS, (t, n, k, pb)
        if k == 0:
            oinfo, pt, po, oipiv, mg = orc.getrf(A.copy(order="F"), 32, 32, margins=True)
            gip = vb.ipiv_t[t][:n].cpu().numpy().astype(np.int64)
            robust = mg > 1 + 1e3 * n * EPS
            assert np.array_equal(gip[robust], oipiv[robust]), (t, n, pb)


@pytest.mark.parametrize("tier,pb", [("fp32", 16), ("fp32", 32), ("fp64", 32)])
def test_vbatched_mixed_tiers(orc, slt, monkeypatch, tier, pb):
    """The mixed API in each tier the table can pick: FP32 factor + FP64
    refinement (iter >= 0) or the direct FP64 solve of a copy (iter 0);
    A and B untouched either way."""
    import torch
    monkeypatch.setenv("SLT_VBATCHED_TIER", tier)
    monkeypatch.setenv("SLT_VBATCHED_PB", str(pb))
    systems = _systems(orc, [1, 16, 31, 64, 97, 200], 8)
    dsys = _to_dev_systems(slt, systems)
    X = [slt.colmajor(torch.zeros_like(b)) for _, _, b in dsys]
    vb = slt.VBatch(dsys, X=X)
    info, it = slt.solve_mixed_vbatched(vb, slt.Options())
    torch.cuda.synchronize()
    assert (info == 0).all()
    assert ((it == 0).all() if tier == "fp64" else (it >= 0).all()), it
    for t, ((k, A, B), (_, dA, dB), x) in enumerate(zip(systems, dsys, X)):
        n = A.shape[0]
        bar = 3 * EPS if tier == "fp64" else 3 * n * EPS
        assert berr(orc, A, to_host(x), B, sym=(k == 1)) <= bar, (t, n, k)
        assert np.array_equal(to_host(dA), A) and np.array_equal(to_host(dB), B)


def test_vbatched_large_sizes_match_oracle(orc, slt):
    """Sizes across the tuning table's switch to 32-wide panels and up to
    config 5's largest (1024): every system's backward error and, for LU,
    its pivots on rows with a clear margin, against the oracle."""
    import torch
    systems = _systems(orc, [511, 512, 513, 640, 777, 1000, 1024], 11, nrhs_max=4, kinds=[0, 1, 0, 1, 0, 0, 1])
    dsys = _to_dev_systems(slt, systems)
    vb = slt.VBatch(dsys)
    info = slt.solve_vbatched(vb)
    torch.cuda.synchronize()
    assert (info == 0).all()
    for t, ((k, A, B), (_, dA, dB)) in enumerate(zip(systems, dsys)):
        n = A.shape[0]
        assert berr(orc, A, to_host(dB), B, sym=(k == 1)) <= 3 * EPS, (t, n, k)
        if k == 0:
            oinfo, pt, po, oipiv, mg = orc.getrf(A.copy(order="F"), 32, 32, margins=True)
            gip = vb.ipiv_t[t][:n].cpu().numpy().astype(np.int64)
            robust = mg > 1 + 1e3 * n * EPS
            assert np.array_equal(gip[robust], oipiv[robust]), (t, n)
