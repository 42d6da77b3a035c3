"""Regenerate the golden fixtures in this folder from the SLATE sources.

    python tests/golden/make_golden.py [SLATE_SOURCE_DIR]

* matgen_kinds.json -- the deterministic test matrices SLATE's tester prints
  in test/ref/<kind>.txt (20 x 20, nb 4, 4 significant digits), parsed from
  those files, for the kinds the oracle restates.
* philox.json -- outputs of SLATE's own slate::random::generate
  (matgen/random.cc), compiled from the SLATE sources by oracle/build_ref.sh,
  for a set of (distribution, seed, shape, offset) cases, stored bit-exactly
  as hex of the IEEE bytes.
"""
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
    src = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    import oracle as O
    kinds = {}
    for kind in O.KINDS:
        p = os.path.join(src, "test", "ref", kind + ".txt")
        if os.path.exists(p):
            kinds[kind] = parse_ref(p)
    with open(os.path.join(HERE, "matgen_kinds.json"), "w") as f:
        json.dump({"source": "SLATE test/ref/<kind>.txt (tester --dim 20 --nb 4 --verbose 4 matgen)",
                   "digits": 4, "kinds": kinds}, f)

    subprocess.check_call(["bash", os.path.join(ROOT, "oracle", "build_ref.sh")])
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


if __name__ == "__main__":
    main()
