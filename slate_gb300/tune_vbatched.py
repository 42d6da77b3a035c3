"""Autotuner of the variable-size batched solver; writes vbatched_table.h.

For each size bucket (n in (lo, hi]) it times, on the current GPU, a batch of
seeded random systems (half general, half SPD, 1-8 right-hand sides):

* the FP64 batched solve with panel width 16 and 32;
* the mixed batched solve in the FP32 tier (FP32 factor + FP64 refinement)
  with panel width 16 and 32, and in the FP64 tier (direct FP64 solve of a
  copy, at the FP64 winner's width);

and keeps the fastest choice per bucket.  The kernels read the table when the
library is built, so run ``__graft_entry__.build()`` after regenerating it.

    python -m slate_gb300.tune_vbatched [--out PATH] [--reps 3] [--scale 1.0]

Per-variant choices are forced through SLT_VBATCHED_PB and SLT_VBATCHED_TIER,
which the library reads on every call.
"""
import argparse
import json
import os
import sys

import numpy as np

EDGES = [0, 64, 128, 256, 512, 1024, 2048]
HEADER = os.path.join(os.path.dirname(os.path.abspath(__file__)), "csrc", "vbatched_table.h")


def _bucket_batch(lo, hi, scale, seed):
    """Sizes, right-hand sides and kinds of one bucket's timing batch: about
    1e12 flop or 8 GB of matrices, whichever is smaller, and at least two
    waves of one CTA per SM."""
    rng = np.random.default_rng(seed)
    mean_n = 0.5 * (lo + 1 + hi)
    per = (2.0 / 3.0 + 1.0 / 3.0) / 2 * mean_n ** 3
    by_flops = scale * 1.0e12 / per
    by_bytes = 8.0e9 / (8.0 * mean_n * mean_n)          # FP64 matrices held: about 8 GB per copy
    cnt = int(np.clip(min(by_flops, by_bytes), 304, 40000))
    ns = rng.integers(lo + 1, hi + 1, cnt)
    rs = rng.integers(1, 9, cnt)
    kinds = np.arange(cnt) % 2
    return ns, rs, kinds


class _Batch:
    def __init__(self, torch, slt, ns, rs, kinds, seed):
        dev = torch.device("cuda")
        self.torch = torch
        self.offA = np.concatenate([[0], np.cumsum(ns * ns)])
        self.offB = np.concatenate([[0], np.cumsum(ns * rs)])
        g = torch.Generator(device=dev)
        g.manual_seed(seed)
        self.A0 = torch.randn(int(self.offA[-1]), dtype=torch.float64, device=dev, generator=g)
        self.B0 = torch.randn(int(self.offB[-1]), dtype=torch.float64, device=dev, generator=g)
        for i in np.nonzero(kinds == 1)[0]:
            n = int(ns[i])
            a = self.A0[self.offA[i]:self.offA[i + 1]].view(n, n)
            a.copy_(a @ a.t() / n + torch.eye(n, dtype=torch.float64, device=dev))
        self.A = self.A0.clone()
        self.B = self.B0.clone()
        self.X = torch.zeros_like(self.B0)
        sysv = [(int(kinds[i]), self.A[self.offA[i]:self.offA[i + 1]].view(int(ns[i]), int(ns[i])).t(),
                 self.B[self.offB[i]:self.offB[i + 1]].view(int(rs[i]), int(ns[i])).t()) for i in range(len(ns))]
        Xv = [self.X[self.offB[i]:self.offB[i + 1]].view(int(rs[i]), int(ns[i])).t() for i in range(len(ns))]
        self.vb = slt.VBatch(sysv, X=Xv)

    def reset(self):
        self.A.copy_(self.A0)
        self.B.copy_(self.B0)
        self.X.zero_()


def _time(torch, fn, reset, reps):
    best = float("inf")
    for _ in range(reps + 1):             # first call warms up (module load, graph instantiation)
        reset()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        out = fn()
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1) * 1e-3)
    return best, out


def _with_env(pb=None, tier=None):
    for k in ("SLT_VBATCHED_PB", "SLT_VBATCHED_TIER"):
        os.environ.pop(k, None)
    if pb is not None:
        os.environ["SLT_VBATCHED_PB"] = str(pb)
    if tier is not None:
        os.environ["SLT_VBATCHED_TIER"] = tier


def tune(reps=3, scale=1.0, log=sys.stderr):
    import torch
    import slate_gb300 as slt
    rows = []
    for b in range(1, len(EDGES)):
        lo, hi = EDGES[b - 1], EDGES[b]
        ns, rs, kinds = _bucket_batch(lo, hi, scale, 1000 + b)
        bt = _Batch(torch, slt, ns, rs, kinds, 2000 + b)
        rec = {"max_n": hi, "systems": int(len(ns))}
        t64 = {}
        for pb in (16, 32):
            _with_env(pb=pb)
            t64[pb], info = _time(torch, lambda: slt.solve_vbatched(bt.vb), bt.reset, reps)
            if (info != 0).any():
                raise RuntimeError("FP64 batched solve reported info != 0 in bucket %d" % hi)
        pb64 = min(t64, key=t64.get)
        tmix = {}
        for pb in (16, 32):
            _with_env(pb=pb, tier="fp32")
            tmix[("fp32", pb)], _ = _time(torch, lambda: slt.solve_mixed_vbatched(bt.vb, slt.Options()), bt.reset,
                                          reps)
        _with_env(pb=pb64, tier="fp64")
        tmix[("fp64", pb64)], _ = _time(torch, lambda: slt.solve_mixed_vbatched(bt.vb, slt.Options()), bt.reset, reps)
        _with_env()
        tier, pbm = min(tmix, key=tmix.get)
        rec.update({"fp64_ms": {str(k): v * 1e3 for k, v in t64.items()},
                    "mixed_ms": {"%s/%d" % k: v * 1e3 for k, v in tmix.items()},
                    "pb_fp64": pb64, "mixed_tier": 1 if tier == "fp32" else 0,
                    "pb_mixed": pbm if tier == "fp32" else pb64})
        print(json.dumps(rec), file=log, flush=True)
        rows.append(rec)
        del bt
        torch.cuda.empty_cache()
    return rows


def write_header(rows, path, gpu_name=""):
    lines = [
        "// vbatched_table.h -- per-size-bucket choices of the batched solver.",
        "// Written by slate_gb300/tune_vbatched.py from timings on %s; re-run it" % (gpu_name or "the GPU"),
        "// to regenerate.  For systems with n <= max_n: the panel width of the FP64",
        "// batched factorisation, and for the mixed API the tier (1: FP32 factor +",
        "// FP64 refinement, 0: direct FP64 solve of a copy) and its panel width.",
        "#pragma once",
        "",
        "struct VbTune { int max_n; int pb_fp64; int mixed_tier; int pb_mixed; };",
        "",
        "static const VbTune kVbTable[] = {",
    ]
    for r in rows:
        t64 = "/".join("%.1f" % v for v in r["fp64_ms"].values())
        tm = ", ".join("%s %.1f" % kv for kv in r["mixed_ms"].items())
        lines.append("    {%d, %d, %d, %d},   // %d systems; FP64 pb16/pb32 %s ms; mixed %s ms" %
                     (r["max_n"], r["pb_fp64"], r["mixed_tier"], r["pb_mixed"], r["systems"], t64, tm))
    lines += ["};", ""]
    with open(path, "w") as f:
        f.write("\n".join(lines))


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--out", default=HEADER)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--scale", type=float, default=1.0, help="work per bucket relative to 1e12 flop")
    ap.add_argument("--json", default=None, help="also write the timings here")
    a = ap.parse_args(argv)
    import torch
    rows = tune(a.reps, a.scale)
    write_header(rows, a.out, torch.cuda.get_device_name(0))
    if a.json:
        with open(a.json, "w") as f:
            json.dump(rows, f, indent=1)


if __name__ == "__main__":
    main()
