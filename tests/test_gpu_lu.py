"""LU parity on the GPU (getrf / getrs / gesv) against the oracle.

Pass bar (BASELINE): scaled backward error ||B - A X||_1 / (n ||A||_1 ||X||_1)
<= 3 eps64 and pivot sequences identical to the oracle's wherever the pivot
margin |best| / |second| exceeds 1 + 1e3 n eps (rounding can decide below).
"""
import numpy as np
import pytest

from gpu_util import EPS, berr, to_dev, to_host

pytestmark = pytest.mark.gpu


def _lu_check(orc, slt, m, n, nb, ib, seed=1, engine=0, dist=2):
    import torch
    A = orc.generate(dist, seed, m, n)
    A0 = A.copy(order="F")
    dA = to_dev(A)
    info, ipiv = slt.getrf(dA, slt.Options(nb=nb, ib=ib, gemm_engine=engine))
    torch.cuda.synchronize()
    LU = to_host(dA)
    Ao = A0.copy(order="F")
    oinfo, pt, po, oipiv, mg = orc.getrf(Ao, nb, ib, margins=True)
    assert info == oinfo
    gip = slt.ipiv_to_lapack(ipiv, nb)
    robust = mg > 1 + 1e3 * max(m, n) * EPS
    assert np.array_equal(gip[robust], oipiv[robust]), np.nonzero(gip != oipiv)[0][:10]
    if np.array_equal(gip, oipiv):
        scale = max(1.0, np.abs(Ao).max())
        assert np.abs(LU - Ao).max() <= 1e-9 * scale
    return A0, LU, gip


@pytest.mark.parametrize("m,n,nb,ib", [(1, 1, 4, 4), (7, 7, 4, 2), (64, 64, 16, 8), (100, 100, 32, 16),
                                       (257, 257, 64, 16), (300, 200, 64, 32), (200, 300, 64, 32),
                                       (1000, 1000, 256, 32), (1030, 1030, 512, 64)])
def test_getrf_parity(orc, slt, m, n, nb, ib):
    _lu_check(orc, slt, m, n, nb, ib)


@pytest.mark.parametrize("engine", [1, 2])
def test_getrf_both_fp64_engines(orc, slt, engine):
    _lu_check(orc, slt, 600, 600, 128, 32, seed=9, engine=engine)


@pytest.mark.parametrize("n,nb,nrhs", [(1, 4, 1), (33, 16, 2), (500, 128, 1), (777, 256, 5), (1024, 512, 16),
                                       (1100, 256, 20)])
def test_gesv_backward_error(orc, slt, n, nb, nrhs):
    import torch
    A = orc.generate(2, 100 + n, n, n)
    B = orc.generate(2, 200 + n, n, nrhs)
    dA, dB = to_dev(A), to_dev(B)
    info, ipiv = slt.gesv(dA, dB, slt.Options(nb=nb))
    torch.cuda.synchronize()
    assert info == 0
    X = to_host(dB)
    assert berr(orc, A, X, B) <= 3 * EPS
    # same solution as the oracle's gesv to within conditioning
    Ao, Bo = A.copy(order="F"), B.copy(order="F")
    orc.gesv(Ao, Bo, nb)
    assert np.abs(X - Bo).max() <= 1e-8 * max(1.0, np.abs(Bo).max())


def test_gesv_config1(orc, slt):
    """The reference's CPU-runnable configuration: n=4096, nb=256, 1 RHS,
    A and b uniform(-1,1) from fixed Philox seeds."""
    import torch
    n, nb = 4096, 256
    A = orc.generate(2, 1, n, n)
    B = orc.generate(2, 2, n, 1)
    dA, dB = to_dev(A), to_dev(B)
    info, ipiv = slt.gesv(dA, dB, slt.Options(nb=nb, ib=32))
    torch.cuda.synchronize()
    assert info == 0
    assert berr(orc, A, to_host(dB), B) <= 3 * EPS
    Ao = A.copy(order="F")
    oinfo, pt, po, oipiv, mg = orc.getrf(Ao, nb, 16, margins=True)
    gip = slt.ipiv_to_lapack(ipiv, nb)
    robust = mg > 1 + 1e3 * n * EPS
    assert robust.mean() > 0.99
    assert np.array_equal(gip[robust], oipiv[robust])


def test_getrs_separate(orc, slt):
    import torch
    n, nb = 700, 128
    A = orc.generate(2, 31, n, n)
    B = orc.generate(2, 32, n, 3)
    dA = to_dev(A)
    info, ipiv = slt.getrf(dA, slt.Options(nb=nb))
    dB = to_dev(B)
    slt.getrs(dA, ipiv, dB, slt.Options(nb=nb))
    torch.cuda.synchronize()
    assert berr(orc, A, to_host(dB), B) <= 3 * EPS


def test_singular_info(orc, slt):
    import torch
    # exactly singular: column 37 zero -> U(37,37) = 0, info = 38 (1-based)
    n = 100
    A = orc.generate(2, 5, n, n)
    A[:, 37] = 0.0
    dA = to_dev(A)
    info, ipiv = slt.getrf(dA, slt.Options(nb=32, ib=8))
    Ao = A.copy(order="F")
    oinfo = orc.getrf(Ao, 32, 8)[0]
    assert info == oinfo == 38
    # ones: rank one
    dA = to_dev(orc.generate_kind("ones", 40, 40))
    assert slt.getrf(dA, slt.Options(nb=16, ib=4))[0] == 2
    # zeros
    dA = to_dev(np.zeros((10, 10), order="F"))
    assert slt.getrf(dA, slt.Options(nb=4, ib=2))[0] == 1
    torch.cuda.synchronize()


def test_known_answer_identity_and_ties(orc, slt):
    import torch
    dA = to_dev(np.eye(50))
    info, ipiv = slt.getrf(dA, slt.Options(nb=16, ib=4))
    assert info == 0 and np.array_equal(slt.ipiv_to_lapack(ipiv, 16), np.arange(1, 51))
    assert np.array_equal(to_host(dA), np.eye(50))
    # exact ties: GPU keeps the diagonal on a tie and otherwise the lowest row,
    # SLATE's order with one panel thread
    A = np.asfortranarray(np.array([[1., 0, 0, 0], [3, 1, 0, 0], [3, 0, 1, 0], [3, 0, 0, 1]]))
    dA = to_dev(A)
    info, ipiv = slt.getrf(dA, slt.Options(nb=4, ib=1))
    oinfo, pt, po, oipiv, _ = orc.getrf(A.copy(order="F"), 4, 1, panel_threads=1)
    assert np.array_equal(slt.ipiv_to_lapack(ipiv, 4), oipiv)
    B = np.asfortranarray(np.array([[2., 1], [-2, 1]]))
    info, ipiv = slt.getrf(to_dev(B), slt.Options(nb=2, ib=1))
    assert int(ipiv[0]) == 0
    torch.cuda.synchronize()


def test_float32_getrf(orc, slt):
    import torch
    n, nb = 500, 128
    A = orc.generate(2, 77, n, n, dtype=np.float32)
    dA = to_dev(A)
    info, ipiv = slt.getrf(dA, slt.Options(nb=nb, ib=32))
    torch.cuda.synchronize()
    Ao = A.copy(order="F")
    oinfo, pt, po, oipiv, mg = orc.getrf(Ao, nb, 32, margins=True)
    robust = mg > 1 + 1e3 * n * np.finfo(np.float32).eps
    gip = slt.ipiv_to_lapack(ipiv, nb)
    assert np.array_equal(gip[robust], oipiv[robust])


@pytest.mark.parametrize("thr", [0.5, 0.1])
def test_getrf_pivot_threshold(orc, slt, thr):
    """SLATE's PivotThreshold rule (Tile_getrf.hh:272-289): the diagonal is
    kept when |a_jj| >= threshold * max |a_ij|; pivots equal the oracle's."""
    import torch
    n, nb, ib = 500, 128, 32
    A = orc.generate(2, 81, n, n)
    dA = to_dev(A)
    info, ipiv = slt.getrf(dA, slt.Options(nb=nb, ib=ib, pivot_threshold=thr))
    torch.cuda.synchronize()
    oinfo, pt, po, oipiv, mg = orc.getrf(A.copy(order="F"), nb, ib, threshold=thr, margins=True)
    assert info == oinfo == 0
    gip = slt.ipiv_to_lapack(ipiv, nb)
    robust = mg > 1 + 1e3 * n * EPS
    assert np.array_equal(gip[robust], oipiv[robust])
    full = np.arange(1, n + 1)
    assert (gip != full).sum() < (slt.ipiv_to_lapack(slt.getrf(to_dev(A), slt.Options(nb=nb, ib=ib))[1], nb) != full).sum()


def test_getrf_nopiv_via_threshold_zero(orc, slt):
    """Threshold 0 keeps every diagonal pivot (MethodLU::NoPiv)."""
    import torch
    n, nb = 300, 64
    A = np.asfortranarray(orc.generate(2, 82, n, n) + n * np.eye(n))
    dA = to_dev(A)
    info, ipiv = slt.getrf(dA, slt.Options(nb=nb, pivot_threshold=0.0))
    torch.cuda.synchronize()
    assert info == 0
    assert np.array_equal(slt.ipiv_to_lapack(ipiv, nb), np.arange(1, n + 1))
    LU = to_host(dA)
    L = np.tril(LU, -1) + np.eye(n)
    U = np.triu(LU)
    assert np.abs(L @ U - A).max() <= 1e-12 * np.abs(A).max()


def test_getrf_nopiv_method(orc, slt):
    """Options.method_lu = "N" is MethodLU::NoPiv: identity pivots."""
    import torch
    n, nb = 200, 64
    A = np.asfortranarray(orc.generate(2, 83, n, n) + n * np.eye(n))
    dA = to_dev(A)
    info, ipiv = slt.getrf(dA, slt.Options(nb=nb, method_lu="N"))
    torch.cuda.synchronize()
    assert info == 0 and np.array_equal(slt.ipiv_to_lapack(ipiv, nb), np.arange(1, n + 1))


@pytest.mark.parametrize("m,n,nb", [(600, 600, 128), (700, 450, 64), (333, 333, 96)])
def test_getrf_calu(orc, slt, m, n, nb):
    """MethodLU::CALU on one GPU (SLATE's device path with a one-participant
    tournament): the partial-pivoting panel's pivots, U as partial pivoting
    gives it, L21 recomputed as A21 U11^{-1} from the permuted original rows;
    P A = L U to rounding and the solve reaches backward error <= 3 eps."""
    import torch
    A = orc.generate(2, 84, m, n)
    dA = to_dev(A)
    info, ipiv = slt.getrf(dA, slt.Options(nb=nb, ib=32, method_lu="C"))
    torch.cuda.synchronize()
    assert info == 0
    oinfo, pt, po, oipiv, mg = orc.getrf(A.copy(order="F"), nb, 32, margins=True)
    gip = slt.ipiv_to_lapack(ipiv, nb)
    robust = mg > 1 + 1e3 * max(m, n) * EPS
    assert np.array_equal(gip[robust], oipiv[robust])
    LU = to_host(dA)
    k = min(m, n)
    L = np.tril(LU, -1)[:, :k] + np.eye(m, k)
    U = np.triu(LU)[:k, :]
    PA = A.copy()
    for r in range(k):
        p = gip[r] - 1
        if p != r:
            PA[[r, p], :] = PA[[p, r], :]
    assert np.abs(L @ U - PA).max() <= 1e3 * max(m, n) * EPS * np.abs(A).max()
    # partial pivoting's factors agree to rounding (the pivots are the same)
    dG = to_dev(A)
    slt.getrf(dG, slt.Options(nb=nb, ib=32))
    torch.cuda.synchronize()
    np.testing.assert_allclose(LU, to_host(dG), rtol=0, atol=1e-9 * np.abs(to_host(dG)).max())
    if m == n:
        B = orc.generate(2, 85, n, 2)
        dB = to_dev(B)
        slt.getrs(dA, ipiv, dB, slt.Options(nb=nb))
        torch.cuda.synchronize()
        X = to_host(dB)
        assert np.abs(B - A @ X).sum(0).max() / (n * np.abs(A).sum(0).max() * np.abs(X).sum(0).max()) <= 3 * EPS


def _slate_fixture():
    import json
    import os
    import sys
    gold = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    sys.path.insert(0, gold)
    import make_golden
    return make_golden, json.load(open(os.path.join(gold, "slate_getrf.json")))


def test_getrf_pivots_match_slate_panel_code(orc, slt):
    """Whole-matrix pivots against LUs whose panels are SLATE's own
    tile::getrf (tests/golden/slate_getrf.json, one panel thread: the GPU's
    tie order), wherever the pivot margin exceeds rounding."""
    import torch
    mg, data = _slate_fixture()
    inputs = {name: (A, nb, ib) for name, A, nb, ib in mg.getrf_full_inputs(orc)}
    for c in data["full"]:
        if c["threads"] != 1:
            continue
        A, nb, ib = inputs[c["name"]]
        m, n = A.shape
        dA = to_dev(A)
        info, ipiv = slt.getrf(dA, slt.Options(nb=nb, ib=ib))
        torch.cuda.synchronize()
        assert info == c["info"]
        k = np.arange(min(m, n)) // nb
        sip = (k + np.array(c["piv_tile"])) * nb + np.array(c["piv_off"]) + 1
        gip = slt.ipiv_to_lapack(ipiv, nb)
        margin = orc.getrf(np.asfortranarray(A.copy()), nb, ib, margins=True)[4]
        robust = margin > 1 + 1e3 * max(m, n) * EPS
        assert np.array_equal(gip[robust], sip[robust]), c["name"]


def test_getrf_panel_ties_match_slate_panel_code(orc, slt):
    """Exact ties, a zero column and tiny pivots: one panel on the GPU against
    SLATE's panel code with one thread (bit-exact pivots and info)."""
    import torch
    mg, data = _slate_fixture()
    inputs = {name: (A, nb, ib) for name, A, nb, ib in mg.getrf_panel_inputs(orc)}
    for c in data["panels"]:
        if c["threads"] != 1 or c["name"] not in ("ties", "zerocol", "tiny", "zeros"):
            continue
        A, nb, ib = inputs[c["name"]]
        dA = to_dev(A)
        info, ipiv = slt.getrf(dA, slt.Options(nb=nb, ib=ib, pivot_threshold=c["threshold"]))
        torch.cuda.synchronize()
        assert info == c["info"], (c["name"], c["threshold"])
        rel = ipiv.cpu().numpy().astype(np.int64)
        srel = np.array(c["piv_tile"]) * nb + np.array(c["piv_off"])
        assert np.array_equal(rel, srel), (c["name"], c["threshold"], rel[:8], srel[:8])
