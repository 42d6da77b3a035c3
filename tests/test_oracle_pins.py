"""Pin the oracle against SLATE's own outputs (no GPU).

* Philox: bit-exact against fixtures produced by SLATE's matgen/random.cc
  (tests/golden/philox.json), and against that code itself when
  oracle/_ref/ has been built from the SLATE sources.
* Deterministic generators: against the tester's printed matrices in SLATE's
  test/ref/*.txt (tests/golden/matgen_kinds.json, 4 significant digits).
"""
import json
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_philox_fixtures_bit_exact(orc):
    data = json.load(open(os.path.join(GOLD, "philox.json")))
    assert len(data["cases"]) >= 100
    for c in data["cases"]:
        dt = np.float64 if c["dtype"] == "f8" else np.float32
        a = orc.generate(c["dist"], c["seed"], c["m"], c["n"], c["ioff"], c["joff"], dtype=dt)
        assert a.tobytes(order="F").hex() == c["hex"], c


def test_philox_against_reference_build(orc):
    if orc.ref_lib() is None:
        pytest.skip("oracle/_ref not built (SLATE sources absent on this host)")
    rng = np.random.default_rng(7)
    for _ in range(20):
        dist = int(rng.integers(1, 8))
        seed = int(rng.integers(0, 2**62))
        m, n = int(rng.integers(1, 40)), int(rng.integers(1, 40))
        io, jo = int(rng.integers(0, 2**40)), int(rng.integers(0, 2**40))
        for dt in (np.float64, np.float32):
            a = orc.generate(dist, seed, m, n, io, jo, dtype=dt)
            b = orc.ref_generate(dist, seed, m, n, io, jo, dtype=dt)
            assert a.tobytes(order="F") == b.tobytes(order="F")


def test_philox_known_state(orc):
    # the all-zero counter under key 0 is fixed by the round function alone
    a = orc.philox(0, 0, 0)
    b = orc.philox(0, 0, 0)
    assert a == b and a != (0, 0)


def _printed(x):
    """The value as SLATE's print_matrix shows it: 4 decimals for |x| >= 0.01,
    4 significant digits below."""
    return np.vectorize(lambda v: float("%.4f" % v) if abs(v) >= 0.01 or v == 0 else float("%.4g" % v))(x)


@pytest.mark.parametrize("kind", ["zeros", "ones", "identity", "ij", "jordan", "jordanT", "kms",
                                  "minij", "hilb", "lehmer", "lotkin"])
def test_deterministic_kinds_match_reference_prints(orc, kind):
    data = json.load(open(os.path.join(GOLD, "matgen_kinds.json")))
    ref = np.array(data["kinds"][kind])
    assert ref.shape == (20, 20)
    a = orc.generate_kind(kind, 20, 20)
    np.testing.assert_allclose(_printed(a), ref, rtol=1e-12, atol=1e-12)


# ---------------------------------------------------------------------------
# LU panel: the oracle's restatement against SLATE's own tile::getrf
# (src/internal/Tile_getrf.hh), compiled from the SLATE sources.
def _getrf_inputs(orc):
    import sys
    sys.path.insert(0, GOLD)
    import make_golden
    return make_golden


def test_getrf_panel_fixtures_bit_exact(orc):
    """Pivots, info and the factored panel (bit for bit) of SLATE's panel
    code, for Philox panels and edge cases, under 1, 2 and 4 panel threads
    and thresholds 1, 0.5 and 0."""
    import hashlib
    mg = _getrf_inputs(orc)
    data = json.load(open(os.path.join(GOLD, "slate_getrf.json")))
    inputs = {name: (A, nb, ib) for name, A, nb, ib in mg.getrf_panel_inputs(orc)}
    assert len(data["panels"]) >= 90
    for c in data["panels"]:
        A, nb, ib = inputs[c["name"]]
        P = np.asfortranarray(A.copy())
        info, pt, po, _, _ = orc.getrf(P, nb, ib, panel_threads=c["threads"], threshold=c["threshold"])
        key = (c["name"], c["threads"], c["threshold"])
        assert info == c["info"], key
        assert pt.tolist() == c["piv_tile"] and po.tolist() == c["piv_off"], key
        assert hashlib.sha256(P.tobytes(order="F")).hexdigest() == c["factor_sha256"], key


def test_getrf_full_fixtures_pivots(orc):
    """Whole-matrix pivot sequences of LUs whose panels are SLATE's."""
    mg = _getrf_inputs(orc)
    data = json.load(open(os.path.join(GOLD, "slate_getrf.json")))
    inputs = {name: (A, nb, ib) for name, A, nb, ib in mg.getrf_full_inputs(orc)}
    for c in data["full"]:
        A, nb, ib = inputs[c["name"]]
        info, pt, po, _, _ = orc.getrf(np.asfortranarray(A.copy()), nb, ib, panel_threads=c["threads"])
        assert info == c["info"]
        assert pt.tolist() == c["piv_tile"] and po.tolist() == c["piv_off"], (c["name"], c["threads"])


def test_getrf_panel_against_reference_build(orc):
    """Random panels against SLATE's panel code itself, where it was built."""
    if orc.ref_getrf_lib() is None:
        pytest.skip("oracle/_ref not built (SLATE sources absent on this host)")
    rng = np.random.default_rng(11)
    for t in range(40):
        nb = int(rng.choice([8, 16, 32, 48]))
        m = int(rng.integers(1, 5)) * nb + int(rng.integers(0, nb))
        ib = int(rng.choice([4, 8, 16, nb]))
        thr = float(rng.choice([1.0, 0.5, 0.1, 0.0]))
        T = int(rng.integers(1, 5))
        A = orc.generate(int(rng.choice([1, 2, 3])), 900 + t, m, nb)
        if t % 5 == 0:
            A = np.asfortranarray(np.round(A * 2))          # exact ties
        rinfo, rpt, rpo, R = orc.ref_getrf_panel(A, nb, ib, thr, T)
        P = np.asfortranarray(A.copy())
        info, pt, po, _, _ = orc.getrf(P, nb, ib, panel_threads=T, threshold=thr)
        assert info == rinfo and np.array_equal(pt, rpt) and np.array_equal(po, rpo), (t, m, nb, ib, thr, T)
        assert np.array_equal(P, R), (t, m, nb, ib, thr, T)
