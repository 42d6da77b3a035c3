"""Host side of the batched solver's autotuner: the bucket batches it times
stay within their memory bound, and the header it writes is the table the
library compiles (one row per bucket, increasing max_n up to the size limit)."""
import re

import numpy as np

from slate_gb300 import tune_vbatched as tv


def test_bucket_batches_bounded():
    for b in range(1, len(tv.EDGES)):
        lo, hi = tv.EDGES[b - 1], tv.EDGES[b]
        ns, rs, kinds = tv._bucket_batch(lo, hi, 1.0, b)
        assert ns.min() > lo and ns.max() <= hi
        assert rs.min() >= 1 and rs.max() <= 8
        assert set(np.unique(kinds)) <= {0, 1}
        assert 304 <= len(ns) <= 40000
        assert 8.0 * float((ns.astype(np.float64) ** 2).sum()) <= 12e9


def _parse(text):
    return [tuple(int(v) for v in m) for m in
            re.findall(r"\{(\d+), (\d+), (\d+), (\d+)\}", text)]


def test_header_roundtrip(tmp_path):
    rows = [{"max_n": hi, "systems": 10, "fp64_ms": {"16": 1.0, "32": 2.0},
             "mixed_ms": {"fp32/16": 1.5, "fp32/32": 1.2, "fp64/16": 1.1},
             "pb_fp64": 16, "mixed_tier": 0, "pb_mixed": 16} for hi in tv.EDGES[1:]]
    p = tmp_path / "t.h"
    tv.write_header(rows, str(p), "GPU")
    assert _parse(p.read_text()) == [(hi, 16, 0, 16) for hi in tv.EDGES[1:]]


def test_committed_table_is_valid():
    with open(tv.HEADER) as f:
        rows = _parse(f.read())
    assert [r[0] for r in rows] == tv.EDGES[1:]
    for max_n, pb64, tier, pbm in rows:
        assert pb64 in (16, 32) and pbm in (16, 32) and tier in (0, 1)


# ---------------------------------------------------------------------------
# single-system driver table (slate_gb300/tune_drivers.py -> csrc/driver_table.h)
from slate_gb300 import tune_drivers as td


def _parse_drivers(text):
    rows = re.findall(r"\{(\d), (\d), (int64_t\(1\) << 62|\d+), (\d+), (\d)(?:, (\d))?\}", text)
    return [(int(k), int(c), (1 << 62) if "<<" in m else int(m), int(p), int(e), int(d) if d else 1)
            for k, c, m, p, e, d in rows]


def test_driver_header_roundtrip(tmp_path):
    rows = [(0, 0, 2048, 19, 1, 1, {(0, 1, 1): 0.1, (19, 1, 1): 0.08}), (0, 0, 4096, 10, 2, 1, {(10, 2, 1): 0.2}),
            (1, 2, 8192, 0, 1, 4, {(0, 1, 1): 0.3, (0, 1, 4): 0.2})]
    p = tmp_path / "d.h"
    td.write(rows, str(p))
    assert _parse_drivers(p.read_text()) == [(0, 0, 2048, 19, 1, 1), (0, 0, 1 << 62, 10, 2, 1),
                                             (1, 2, 1 << 62, 0, 1, 4)]


def test_committed_driver_table_is_valid():
    with open(td.HEADER) as f:
        rows = _parse_drivers(f.read())
    keys = {(k, c) for k, c, _, _, _, _ in rows}
    assert keys == {(k, c) for k in (0, 1) for c in (0, 1, 2)}
    for key in keys:
        group = [r for r in rows if (r[0], r[1]) == key]
        assert [r[2] for r in group] == sorted(r[2] for r in group)
        assert group[-1][2] == 1 << 62                  # the last bucket takes every larger n
    for k, _, _, p, e, d in rows:
        assert 0 <= p < 152 and e in (1, 2) and d in (1, 2, 4, 8)
        assert d == 1 or (k == 1 and p == 0)          # deferred updates: potrf without overlap
