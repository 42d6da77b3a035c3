"""Autotuner of the single-system factorisations; writes csrc/driver_table.h.

For each kind (getrf, potrf), update class (FP64; FP32 SIMT; tensor cores, run
in the FP16 tier) and size bucket it times, on the current GPU, one
factorisation of a seeded matrix for every candidate

* SMs given to the panel while the previous step's trailing update runs
  beside it (0 = no overlap; the rest of the SMs go to the update);
* for FP64, the update engine (1 DFMA, 2 DMMA);
* for potrf without overlap, the panels per deferred trailing update
  (1, 2, 4 or 8: the trailing matrix is read and written once per that many
  panels);

and keeps the fastest per bucket.  The library reads the table when it is
built, so run ``__graft_entry__.build()`` after regenerating it.

    python -m slate_gb300.tune_drivers [--out PATH] [--reps 2] [--quick]

The candidates are forced through SLT_LOOKAHEAD_PANEL_SMS and
SLT_UPDATE_DEPTH (read by the library on every call) and Options.gemm_engine.
"""
import argparse
import os
import sys
import time

HEADER = os.path.join(os.path.dirname(os.path.abspath(__file__)), "csrc", "driver_table.h")

PANEL_SMS = [0, 10, 19, 38, 57]
DEPTHS = [2, 4, 8]
SIZES = {
    (0, 0): [2048, 4096, 8192, 16384],
    (0, 1): [4096, 8192, 16384, 32768],
    (0, 2): [4096, 8192, 16384, 32768],
    (1, 0): [2048, 4096, 8192, 16384],
    (1, 1): [4096, 8192, 16384, 32768],
    (1, 2): [8192, 16384, 32768, 65536],
}
CLASS_NAME = {0: "FP64", 1: "FP32 SIMT", 2: "tensor-core (FP16)"}


def _time(torch, fn, reps):
    best = None
    for _ in range(reps):
        torch.cuda.synchronize()
        t = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        dt = time.perf_counter() - t
        best = dt if best is None else min(best, dt)
    return best


def tune(reps=2, quick=False, log=print):
    import torch
    import slate_gb300 as slt
    dev = torch.device("cuda")
    rows = []
    for (kind, cls), sizes in SIZES.items():
        if quick:
            sizes = sizes[:2]
        for n in sizes:
            dt = torch.float64 if cls == 0 else torch.float32
            A0 = slt.colmajor(torch.empty(n, n, dtype=torch.float64, device=dev))
            if kind == 0:
                slt.generate(2, 7, A0)
            else:
                slt.generate_sigma(A0, 10.0, "logrand", True, seed=7)
            A0 = slt.colmajor(A0.to(dt))
            A = slt.colmajor(A0.clone())
            prec = {0: "fp64", 1: "fp32", 2: "fp16"}[cls]
            engines = [1, 2] if cls == 0 else [1]
            results = {}
            cands = [(p, e, 1) for e in engines for p in PANEL_SMS]
            if kind == 1:
                cands += [(0, e, d) for e in engines for d in DEPTHS]
            for p, e, d in cands:
                os.environ["SLT_LOOKAHEAD_PANEL_SMS"] = str(p)
                os.environ["SLT_UPDATE_DEPTH"] = str(d)
                o = slt.Options(nb=512, ib=32, factor_precision=prec, gemm_engine=e)

                def run():
                    A.copy_(A0)
                    info = slt.getrf(A, o)[0] if kind == 0 else slt.potrf(A, o)
                    assert info == 0, info

                run()
                results[(p, e, d)] = _time(torch, run, reps)
            os.environ.pop("SLT_LOOKAHEAD_PANEL_SMS", None)
            os.environ.pop("SLT_UPDATE_DEPTH", None)
            best = min(results, key=results.get)
            rows.append((kind, cls, n, best[0], best[1], best[2], results))
            log("%s %s n=%d: best panel_sms=%d engine=%d depth=%d (%s)" % (
                "getrf" if kind == 0 else "potrf", CLASS_NAME[cls], n, best[0], best[1], best[2],
                ", ".join("%d/%d/%d %.1f ms" % (p, e, d, t * 1e3) for (p, e, d), t in sorted(results.items()))))
            del A, A0
            torch.cuda.empty_cache()
    return rows


def write(rows, path=HEADER):
    lines = ["// driver_table.h -- per-size-bucket choices of the single-system drivers.",
             "// Written by slate_gb300/tune_drivers.py from timings on NVIDIA GB300; re-run",
             "// it to regenerate.  For a factorisation of order n <= max_n of kind (0 getrf,",
             "// 1 potrf) and update class (0 FP64, 1 FP32 SIMT, 2 tensor cores: TF32 /",
             "// BF16 / FP16 / FP8 / 3xTF32): the SMs given to the panel while the rest of",
             "// the previous step's trailing update runs beside it (0: no overlap) and the",
             "// FP64 update engine (1 DFMA with 64 x 64 tiles, 2 DMMA m16n8k4) and, for potrf",
             "// without overlap, the panels per deferred trailing update.  The tile size nb",
             "// stays the caller's (Option::BlockSize): the pivot format of getrf and getrs",
             "// depends on it.  Timings: panel SMs / engine / depth, one factorisation, nb 512.",
             "#pragma once",
             "",
             "#include <cstdint>",
             "",
             "struct DriverTune { int kind; int cls; int64_t max_n; int panel_sms; int engine; int depth; };",
             "",
             "static const DriverTune kDriverTable[] = {"]
    by = {}
    for r in rows:
        by.setdefault((r[0], r[1]), []).append(r)
    for key in sorted(by):
        group = sorted(by[key], key=lambda r: r[2])
        for i, (kind, cls, n, p, e, d, res) in enumerate(group):
            mx = "int64_t(1) << 62" if i == len(group) - 1 else "%d" % n
            times = ", ".join("%d/%d/%d %.1f" % (pp, ee, dd, t * 1e3) for (pp, ee, dd), t in sorted(res.items()))
            lines.append("    {%d, %d, %s, %d, %d, %d},   // %s %s n=%d: %s ms" % (
                kind, cls, mx, p, e, d, "getrf" if kind == 0 else "potrf", CLASS_NAME[cls], n, times))
    lines.append("};")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=HEADER)
    ap.add_argument("--reps", type=int, default=2)
    ap.add_argument("--quick", action="store_true", help="two sizes per class")
    a = ap.parse_args()
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    rows = tune(a.reps, a.quick, log=lambda s: print(s, flush=True))
    write(rows, a.out)
    print("wrote", a.out)


if __name__ == "__main__":
    main()
