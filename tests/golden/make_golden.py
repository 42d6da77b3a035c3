"""Regenerate the golden fixtures in this folder from the SLATE sources.

    python tests/golden/make_golden.py SLATE_SOURCE_DIR   (or SLATE_SRC=... in the environment)

* matgen_kinds.json -- the deterministic test matrices SLATE's tester prints
  in test/ref/<kind>.txt (20 x 20, nb 4, 4 significant digits), parsed from
  those files, for the kinds the oracle restates.
* philox.json -- outputs of SLATE's own slate::random::generate
  (matgen/random.cc), compiled from the SLATE sources by oracle/build_ref.sh,
  for a set of (distribution, seed, shape, offset) cases, stored bit-exactly
  as hex of the IEEE bytes.
* slate_getrf.json -- outputs of SLATE's own tile LU panel
  (src/internal/Tile_getrf.hh, built by oracle/build_ref.sh): pivots, info
  and the factored panel (SHA-256 of its IEEE bytes) for panels of Philox
  inputs and edge cases (exact ties, a zero column, entries near and below
  the safe minimum, an all-zero panel) under 1-4 panel threads and pivot
  thresholds 1, 0.5 and 0; and pivots and info of full LUs whose panels are
  SLATE's (sizes up to 300, nb 64).
"""
import hashlib
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def parse_ref(path):
    rows = []
    inside = False
    for line in open(path):
        s = line.strip()
        if s.startswith("A = ["):
            inside = True
            continue
        if inside:
            if s.startswith("];"):
                break
            if not s:
                continue
            rows.append([float(t) for t in s.split()])
    return rows


def main():
    src = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SLATE_SRC", "")
    if not src or not os.path.isdir(src):
        raise SystemExit("usage: make_golden.py SLATE_SOURCE_DIR (or set SLATE_SRC)")
    import oracle as O
    kinds = {}
    for kind in O.KINDS:
        p = os.path.join(src, "test", "ref", kind + ".txt")
        if os.path.exists(p):
            kinds[kind] = parse_ref(p)
    with open(os.path.join(HERE, "matgen_kinds.json"), "w") as f:
        json.dump({"source": "SLATE test/ref/<kind>.txt (tester --dim 20 --nb 4 --verbose 4 matgen)",
                   "digits": 4, "kinds": kinds}, f)

    subprocess.check_call(["bash", os.path.join(ROOT, "oracle", "build_ref.sh"), src])
    if O.ref_lib() is None:
        raise SystemExit("SLATE sources not available: cannot build the reference generator")
    cases = []
    for dist in range(1, 8):
        for seed in (0, 1, 42, 2**40 + 3):
            for (m, n, io, jo) in ((5, 3, 0, 0), (7, 4, 1000, 77), (3, 2, 2**31 + 5, 12345)):
                for dt in ("f8", "f4"):
                    a = O.ref_generate(dist, seed, m, n, io, jo, dtype=np.float64 if dt == "f8" else np.float32)
                    cases.append({"dist": dist, "seed": seed, "m": m, "n": n, "ioff": io, "joff": jo,
                                  "dtype": dt, "hex": a.tobytes(order="F").hex()})
    with open(os.path.join(HERE, "philox.json"), "w") as f:
        json.dump({"source": "SLATE matgen/random.cc slate::random::generate, built by oracle/build_ref.sh",
                   "cases": cases}, f)
    print("wrote", len(kinds), "kinds and", len(cases), "philox cases")
    write_getrf(O)


def getrf_panel_inputs(O):
    """(name, A, nb, ib) of the panel cases; reproducible without SLATE."""
    out = []
    for seed, (m, nb, ib) in enumerate([(64, 16, 4), (200, 32, 8), (97, 16, 16), (33, 32, 32), (130, 24, 8)], 1):
        out.append(("rand%d" % seed, O.generate(2, seed, m, nb), nb, ib))
    rng = np.random.default_rng(0)
    out.append(("ties", np.asfortranarray(rng.integers(-3, 4, size=(96, 16)).astype(float)), 16, 4))
    A = O.generate(2, 7, 80, 16)
    A[:, 5] = 0.0
    out.append(("zerocol", A, 16, 4))
    out.append(("tiny", np.asfortranarray(O.generate(2, 8, 80, 16) * 1e-300), 16, 4))
    A = O.generate(2, 9, 70, 16)
    A[3:, 2] *= 1e-310
    out.append(("subnormal", A, 16, 8))
    out.append(("zeros", np.zeros((50, 8), order="F"), 8, 4))
    return out


def getrf_full_inputs(O):
    return [("lu%d" % s, O.generate(2, 100 + s, m, n), nb, ib)
            for s, (m, n, nb, ib) in enumerate([(300, 300, 64, 16), (257, 190, 64, 32), (128, 300, 64, 16)])]


def write_getrf(O):
    if O.ref_getrf_lib() is None:
        raise SystemExit("SLATE sources not available: cannot build the reference LU panel")
    panels = []
    for name, A, nb, ib in getrf_panel_inputs(O):
        for thr in (1.0, 0.5, 0.0):
            for T in (1, 2, 4):
                info, pt, po, P = O.ref_getrf_panel(A, nb, ib, thr, T)
                panels.append({"name": name, "nb": nb, "ib": ib, "threshold": thr, "threads": T, "info": info,
                               "piv_tile": pt.tolist(), "piv_off": po.tolist(),
                               "factor_sha256": hashlib.sha256(P.tobytes(order="F")).hexdigest()})
    full = []
    for name, A, nb, ib in getrf_full_inputs(O):
        for T in (1, 4):
            info, pt, po, P = O.ref_getrf(A, nb, ib, 1.0, T)
            full.append({"name": name, "m": A.shape[0], "n": A.shape[1], "nb": nb, "ib": ib, "threads": T,
                         "info": info, "piv_tile": pt.tolist(), "piv_off": po.tolist()})
    with open(os.path.join(HERE, "slate_getrf.json"), "w") as f:
        json.dump({"source": "SLATE src/internal/Tile_getrf.hh tile::getrf, built by oracle/build_ref.sh; "
                             "inputs from tests/golden/make_golden.py getrf_panel_inputs / getrf_full_inputs",
                   "panels": panels, "full": full}, f)
    print("wrote", len(panels), "panel cases and", len(full), "full LU cases")


if __name__ == "__main__":
    main()
