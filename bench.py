"""Benchmark: gesv/posv effective TFLOP/s at FP64 backward error, mixed vs
plain FP64, one GB300.

Headline workload (default, BASELINE config 4): posv_mixed_gmres, n = 65536,
nb = 512, 16 right-hand sides; SPD A = Q diag(s) Q^T with s log-uniform in
[1/kappa, 1], kappa = 1e2 (Q orthogonal, Philox-drawn butterfly levels, seed
3), b = A x_true with x_true ~ U(-1,1) (Philox seed 5); FP16 tensor-core
Cholesky, FP64 GMRES-IR to SLATE's stopping test.  One step = one solve with
A and B resident in HBM (A is 34 GB, far above L2, so no flush is needed).
``value`` = LAPACK posv flop count (n^3/3 + n^2/2 + n/6 + 2 n^2 nrhs) / step
time; the plain FP64 posv on the same system is timed once beside it, and
``e2e`` runs the same solve through the LAPACK-compatible host entry point
slate_dsposv (pinned host buffers, host<->device copies inside the timing).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--config 1|2|3|4|5] [--sweep] [--prec fp16|bf16|fp32|...]

--impl reference times the CPU restatement of SLATE's posv_mixed_gmres (the
oracle; SLATE itself cannot be built here) on the host cores, each step one
solve of the same workload family at the largest n whose K + W steps fit the
step budget (the n it ran is in its config).  Under torchrun (N > 1) every
rank solves its own replica ("replicas only": one factorisation does not
shard); value = total solves x flops / max time.

--config 2 prints the same kind of line for BASELINE config 2 (posv_mixed,
n = 16384, 4 RHS, A = G G^T / n + I).  Other records (one JSON line per case):
  1  plain FP64 gesv, n=4096 nb=256, 1 RHS, A and b U(-1,1); pivots and
     backward error against the oracle, the oracle's gesv timed beside it;
  3  gesv_mixed, n=32768 nb=512, 1 RHS, A = U diag(s) V^T with s geometric
     from 1 to 1/kappa, kappa in {1e2, 1e4, 1e6}, FP32/BF16/FP16 factors,
     b = A x_true; plain FP64 gesv timed on the same system;
  4 --sweep  posv_mixed_gmres, n=65536 nb=512, 16 RHS, kappa in {1e2, 1e5,
     1e8}, FP16/BF16 factors; plain FP64 posv timed on the same system;
  5  20000 independent systems, n log-uniform in [32, 1024], 1-8 RHS, half
     general (U(-1,1), LU) and half SPD (G G^T/n + I, Cholesky): the batched
     FP64 solve and the batched FP32-factor + FP64-refinement solve (one
     launch each plus the refinement graph) against a loop of per-system
     gesv / posv calls.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)


def posv_flops(n, nrhs):
    return n**3 / 3.0 + n**2 / 2.0 + n / 6.0 + 2.0 * n**2 * nrhs


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--config", type=int, default=4, choices=[1, 2, 3, 4, 5])
    p.add_argument("--sweep", action="store_true", help="config 4: kappa x precision records")
    p.add_argument("--prec", default="fp16")
    p.add_argument("--n", type=int, default=None, help="matrix order (default: the config's)")
    p.add_argument("--nb", type=int, default=512)
    p.add_argument("--nrhs", type=int, default=None, help="right-hand sides (default: the config's)")
    p.add_argument("--kappa", type=float, default=1e2, help="headline condition number (config 4)")
    p.add_argument("--cpu-n", type=int, default=None, help="CPU sample size (default: fit the budget)")
    p.add_argument("--cpu-budget", type=float, default=150.0,
                   help="seconds of CPU work the reference arm's W + K steps may take")
    p.add_argument("--e2e-steps", type=int, default=3, help="timed steps of the end-to-end leg")
    p.add_argument("--no-plain", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--batch", type=int, default=20000, help="config 5: number of systems")
    p.add_argument("--no-loop", action="store_true", help="config 5: skip the per-system loop")
    p.add_argument("--kappas", default=None, help="comma list (configs 3, 4 --sweep)")
    p.add_argument("--precs", default=None, help="comma list (configs 3, 4 --sweep)")
    p.add_argument("--refine", default="ir+gmres", help="configs 3: ir | ir+gmres")
    p.add_argument("--residual-engine", type=int, default=0,
                   help="FP64 residuals: 0 auto, 1 FP64 FMA, 2 tensor-core digit products")
    a = p.parse_args()
    w = WORKLOADS.get(a.config)
    if w is not None:
        a.n = a.n or w["n"]
        a.nrhs = a.nrhs or w["nrhs"]
    return a


# The headline workloads (BASELINE configs 4 and 2).  "sigma": SPD
# Q diag(s) Q^T, s log-uniform in [1/kappa, 1] (SLATE's poev + logrand);
# "ggt": G G^T / n + I with G ~ N(0,1).
WORKLOADS = {
    4: {"routine": "posv_mixed_gmres", "n": 65536, "nrhs": 16, "matrix": "sigma"},
    2: {"routine": "posv_mixed", "n": 16384, "nrhs": 4, "matrix": "ggt"},
}

METRIC = "gesv/posv effective TFLOP/s at FP64 backward error: mixed vs plain FP64, 1 GB300"


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Clocks:
    """nvidia-smi samples during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "50"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        out, _ = self.p.communicate(timeout=10)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_headline_system(slt, torch, args, device):
    """The headline system on the device: A, B = A x_true (or B ~ U(-1,1)
    for the ggt matrix) and x_true (None for ggt)."""
    w = WORKLOADS[args.config]
    n, nrhs = args.n, args.nrhs
    if w["matrix"] == "ggt":
        A, B = make_system(slt, torch, n, nrhs, device)
        return A, B, None
    A = slt.colmajor(torch.empty(n, n, dtype=torch.float64, device=device))
    slt.generate_sigma(A, args.kappa, "logrand", True, seed=3)
    Xt = slt.colmajor(torch.empty(n, nrhs, dtype=torch.float64, device=device))
    slt.generate(2, 5, Xt)
    B = slt.colmajor(A @ Xt)        # cuBLAS FP64: set-up of the right-hand side, outside any timing
    torch.cuda.synchronize()
    return A, B, Xt


def make_system(slt, torch, n, nrhs, device):
    """A = G G^T / n + I (G from SLATE's Philox normal stream), B ~ U(-1,1)."""
    G = slt.colmajor(torch.empty(n, n, dtype=torch.float64, device=device))
    slt.generate(3, 1, G)
    Gf = G.to(torch.float32)
    del G
    torch.backends.cuda.matmul.allow_tf32 = False
    S = (Gf @ Gf.t()) / n
    del Gf
    A = S.to(torch.float64)
    del S
    A.diagonal().add_(1.0)
    A = slt.colmajor(A)             # symmetric: column-major view of the same values
    B = slt.colmajor(torch.empty(n, nrhs, dtype=torch.float64, device=device))
    slt.generate(2, 2, B)
    torch.cuda.synchronize()
    return A, B


def backward_error(torch, A, X, B):
    """||B - A X||_1 / (n ||A||_1 ||X||_1) (SLATE tester, test/test_posv.cc)."""
    n = A.shape[0]
    R = B - A @ X
    an = A.abs().sum(0).max()
    return float(R.abs().sum(0).max() / (n * an * X.abs().sum(0).max()))


def _oracle_setup():
    # one BLAS thread per tile task, as SLATE's HostTask runs tile BLAS inside
    # OpenMP tasks (nested BLAS threads would oversubscribe the cores)
    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    cores = os.cpu_count() or 1
    oracle.set_threads(cores)
    blas = oracle.use_host_blas()
    return oracle, cores, blas


def _oracle_system(oracle, args, n):
    """The headline workload family at order n on the host."""
    w = WORKLOADS[args.config]
    if w["matrix"] == "ggt":
        G = oracle.generate(3, 1, n, n)
        A = np.asfortranarray(G @ G.T / n + np.eye(n))
        return A, oracle.generate(2, 2, n, args.nrhs)
    A = oracle.generate_sigma(n, args.kappa, "logrand", True, 3)
    Xt = oracle.generate(2, 5, n, args.nrhs)
    return A, np.asfortranarray(A @ Xt)


def _oracle_solve(oracle, args, A, B):
    """One solve of the headline routine by the oracle; returns (info, iter)."""
    if WORKLOADS[args.config]["routine"] == "posv_mixed_gmres":
        info, X, it, _ = oracle.posv_mixed_gmres_nrhs(A, B, args.nb)
    else:
        info, X, it = oracle.posv_mixed(A, B, args.nb)
    return info, it


def _cpu_sample_n(oracle, args, budget_s, steps):
    """The largest n (a multiple of 1024, at most the workload's) whose
    `steps` solves fit in budget_s seconds, from one timed probe solve
    scaled by n^3."""
    if args.cpu_n:
        return min(args.cpu_n, args.n), None
    n0 = min(4096, args.n)
    A, B = _oracle_system(oracle, args, n0)
    t = time.perf_counter()
    _oracle_solve(oracle, args, A, B)
    t0 = time.perf_counter() - t
    per = budget_s / max(1, steps)
    n = int(n0 * (per / max(t0, 1e-6)) ** (1.0 / 3.0)) // 1024 * 1024
    return max(min(n, args.n, 32768), n0), t0


def run_reference(args):
    """The CPU restatement of SLATE's solver on the host cores (rank 0 only)."""
    ws, rank, local = dist_env()
    if rank != 0:
        return
    oracle, cores, blas = _oracle_setup()
    n, probe = _cpu_sample_n(oracle, args, args.cpu_budget, args.warmup + args.steps)
    A, B = _oracle_system(oracle, args, n)
    times, it, info = [], 0, 0
    for i in range(args.warmup + args.steps):
        Aw = A.copy(order="F")
        t = time.perf_counter()
        info, it = _oracle_solve(oracle, args, Aw, B)
        dt = time.perf_counter() - t
        if i >= args.warmup:
            times.append(dt)
    t = statistics.median(times)
    val = posv_flops(n, args.nrhs) / t / 1e12
    w = WORKLOADS[args.config]
    sample = ("%s restatement (the oracle, SLATE's algorithm; GMRES per column sharing one factorisation) "
              "at n=%d nb=%d nrhs=%d, the same matrix family as the GPU workload at a size whose %d steps "
              "fit the run's CPU budget; host BLAS %s" % (w["routine"], n, args.nb, args.nrhs,
                                                          args.warmup + args.steps,
                                                          "scipy-openblas" if blas else "built-in"))
    cfg = config(args, n=n)
    cfg["sample_of"] = "n=%d" % args.n
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": "TFLOP/s",
            "higher_is_better": True, "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t * 1e3, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": cfg,
            "cpu_baseline": {"value": val, "unit": "TFLOP/s", "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": val, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "iter": it, "info": info}
    print(json.dumps(line))


def config(args, n=None):
    n = n or args.n
    w = WORKLOADS[args.config]
    if w["matrix"] == "sigma":
        mat = ("SPD A = Q diag(s) Q^T, s log-uniform in [1/kappa, 1], kappa=%g (poev+logrand; Q from "
               "Philox butterfly levels, seed 3), B = A x_true, x_true U(-1,1) seed 5" % args.kappa)
    else:
        mat = "A = G G^T/n + I (G Philox N(0,1), seed 1), B U(-1,1) seed 2"
    return {"workload": "%s n=%d nb=%d nrhs=%d, %s, %s factor" % (w["routine"], n, args.nb, args.nrhs, mat,
                                                                args.prec.upper()),
            "routine": w["routine"], "n": n, "nb": args.nb, "nrhs": args.nrhs, "factor_precision": args.prec,
            "kappa": args.kappa if w["matrix"] == "sigma" else None,
            "l2": "inputs larger than L2 (A is %.1f GB)" % (8.0 * n * n / 1e9),
            "parallelism": "replicas x%d" % args.gpus}


def cpu_baseline_sample(args):
    """Oracle solve on the host cores, a bounded sample (about 10-30 s of
    CPU work), rank 0 at N=1."""
    oracle, cores, blas = _oracle_setup()
    n, _ = _cpu_sample_n(oracle, args, 20.0, 1)
    A, B = _oracle_system(oracle, args, n)
    t = time.perf_counter()
    info, it = _oracle_solve(oracle, args, A, B)
    dt = time.perf_counter() - t
    return {"value": posv_flops(n, args.nrhs) / dt / 1e12, "unit": "TFLOP/s", "cores": cores, "kind": "port",
            "sample": "%s restatement at n=%d nb=%d nrhs=%d, same matrix family (%.1f s, %d iterations), "
                      "host BLAS %s" % (WORKLOADS[args.config]["routine"], n, args.nb, args.nrhs, dt, it,
                                        "scipy-openblas" if blas else "built-in")}


def gesv_flops(n, nrhs):
    return 2.0 * n**3 / 3.0 - n**2 / 2.0 + 5.0 * n / 6.0 + 2.0 * n**2 * nrhs


def _event_time(torch, fn):
    """Seconds of fn() between CUDA events on the current stream."""
    st = torch.cuda.current_stream()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record(st)
    r = fn()
    b.record(st)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / 1e3, r


def _rel_fwd(torch, X, Xt):
    return float((X - Xt).abs().max() / Xt.abs().max())


def run_config1(args, slt, torch, dev):
    """Plain FP64 gesv n=4096 nb=256 (SLATE's HostTask tester configuration)."""
    n, nb, nrhs = 4096, 256, 1
    A0 = slt.colmajor(torch.empty(n, n, dtype=torch.float64, device=dev))
    B0 = slt.colmajor(torch.empty(n, nrhs, dtype=torch.float64, device=dev))
    slt.generate(2, 1, A0)
    slt.generate(2, 2, B0)
    A = slt.colmajor(A0.clone())
    B = slt.colmajor(B0.clone())
    opts = slt.Options(nb=nb, ib=32)
    times = []
    for i in range(args.warmup + args.steps):
        A.copy_(A0)
        B.copy_(B0)
        t, (info, ipiv) = _event_time(torch, lambda: slt.gesv(A, B, opts))
        if i >= args.warmup:
            times.append(t)
    t = statistics.median(times)
    berr = backward_error(torch, A0, B, B0)
    rec = {"config": 1, "workload": "gesv n=4096 nb=256 nrhs=1, A, b Philox U(-1,1) seeds 1, 2",
           "dtype": "f64", "steps": args.steps, "warmup": args.warmup, "ms": t * 1e3,
           "tflops": gesv_flops(n, nrhs) / t / 1e12, "getrf_ms": slt.timer("gesv::getrf") * 1e3,
           "info": info, "backward_error": berr, "bound_3eps": 3 * np.finfo(np.float64).eps}
    if not args.no_cpu:
        os.environ["OPENBLAS_NUM_THREADS"] = "1"
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        oracle.build()
        cores = os.cpu_count() or 1
        oracle.set_threads(cores)
        oracle.use_host_blas()
        Ah = oracle.generate(2, 1, n, n)
        Bh = oracle.generate(2, 2, n, nrhs)
        t0 = time.perf_counter()
        oinfo, pt, po = oracle.gesv(Ah, Bh, nb)
        tc = time.perf_counter() - t0
        k = np.arange(n) // nb
        oip = (k + pt) * nb + po + 1                      # LAPACK ipiv of the oracle's pivots
        gip = np.asarray(slt.ipiv_to_lapack(ipiv, nb)).astype(np.int64)
        rec["cpu_baseline"] = {"ms": tc * 1e3, "tflops": gesv_flops(n, nrhs) / tc / 1e12, "cores": cores,
                               "kind": "port", "sample": "oracle gesv, same n and inputs"}
        rec["pivot_mismatches_vs_oracle"] = int(np.count_nonzero(oip != gip))
        rec["solution_max_diff_vs_oracle"] = float(np.abs(Bh[:, 0] - B.cpu().numpy()[:, 0]).max())
    print(json.dumps(rec))


def run_mixed_sweep(args, slt, torch, dev, cfg):
    """Configs 3 (gesv_mixed) and 4 (posv_mixed_gmres): kappa x precision."""
    chol = cfg == 4
    n = args.n or (65536 if chol else 32768)
    nb, nrhs = 512, (16 if chol else 1)
    kappas = [float(k) for k in (args.kappas or ("1e2,1e5,1e8" if chol else "1e2,1e4,1e6")).split(",")]
    precs = (args.precs or ("fp16,bf16" if chol else "fp32,bf16,fp16")).split(",")
    fn = slt.posv_mixed_gmres if chol else slt.gesv_mixed
    flops = posv_flops(n, nrhs) if chol else gesv_flops(n, nrhs)
    A0 = slt.colmajor(torch.empty(n, n, dtype=torch.float64, device=dev))
    A = slt.colmajor(torch.empty(n, n, dtype=torch.float64, device=dev))
    Xt = slt.colmajor(torch.empty(n, nrhs, dtype=torch.float64, device=dev))
    slt.generate(2, 5, Xt)
    X = slt.colmajor(torch.zeros(n, nrhs, dtype=torch.float64, device=dev))
    plain_t = None
    for kappa in kappas:
        slt.generate_sigma(A0, kappa, "logrand" if chol else "geo", chol, seed=3)
        B = slt.colmajor(A0 @ Xt)         # b = A x_true (cuBLAS FP64, a cross-check product)
        for prec in precs:
            opts = slt.Options(nb=nb, ib=32, factor_precision=prec, refine=args.refine)
            # A is restored before every run: an FP64 fallback overwrites it with its factors
            for _ in range(max(1, min(args.warmup, 1))):
                A.copy_(A0)
                X.zero_()
                fn(A, B, X, opts)
            A.copy_(A0)
            X.zero_()
            t, (info, it, _) = _event_time(torch, lambda: fn(A, B, X, opts))
            rec = {"config": cfg, "routine": "posv_mixed_gmres" if chol else "gesv_mixed", "n": n, "nb": nb,
                   "nrhs": nrhs, "kappa": kappa, "factor_precision": prec,
                   "refine": "gmres" if chol else args.refine, "ms": t * 1e3, "iter": it, "info": info,
                   "effective_tflops": flops / t / 1e12,
                   "factor_ms": slt.timer(("posv_mixed_gmres::potrf_lo" if chol else "gesv_mixed::getrf_lo")) * 1e3,
                   "backward_error": backward_error(torch, A0, X, B), "forward_error": _rel_fwd(torch, X, Xt),
                   "bound_3n_eps": 3 * n * np.finfo(np.float64).eps}
            print(json.dumps(rec), flush=True)
        if plain_t is None and not args.no_plain:
            A2 = A
            A2.copy_(A0)
            X2 = slt.colmajor(B.clone())
            if chol:
                t, info = _event_time(torch, lambda: slt.posv(A2, X2, slt.Options(nb=nb, ib=32)))
                fkey = "posv::potrf"
            else:
                t, (info, _) = _event_time(torch, lambda: slt.gesv(A2, X2, slt.Options(nb=nb, ib=32)))
                fkey = "gesv::getrf"
            fact = slt.timer(fkey)
            fflops = (n**3 / 3.0) if chol else (2.0 * n**3 / 3.0)
            plain_t = t
            print(json.dumps({"config": cfg, "routine": "posv" if chol else "gesv", "n": n, "nb": nb,
                              "nrhs": nrhs, "kappa": kappa, "factor_precision": "fp64", "ms": t * 1e3,
                              "info": info, "tflops": flops / t / 1e12, "factor_ms": fact * 1e3,
                              "factor_tflops": fflops / fact / 1e12,
                              "backward_error": backward_error(torch, A0, X2, B),
                              "forward_error": _rel_fwd(torch, X2, Xt)}), flush=True)
            del X2
        del B


def run_config5(args, slt, torch, dev, ws=1, rank=0):
    """Variable-size batch: batched FP64, batched mixed, per-system loop.
    Under torchrun the systems are split across ranks (longest processing
    time first, slate_gb300.partition); each rank solves its share with one
    batched launch and the slowest rank's time is reported."""
    rng = np.random.default_rng(12345)
    cnt_all = args.batch
    ns_all = np.exp(rng.uniform(np.log(32), np.log(1024), cnt_all)).astype(np.int64)
    rs_all = rng.integers(1, 9, cnt_all)
    kinds_all = (np.arange(cnt_all) % 2).astype(np.int64)        # even: general, odd: SPD
    sel = np.arange(cnt_all)
    if ws > 1:
        from slate_gb300.partition import partition_systems, system_costs
        sel = partition_systems(system_costs(ns_all, rs_all, kinds_all), ws)[0][rank]
    ns, rs, kinds = ns_all[sel], rs_all[sel], kinds_all[sel]
    cnt = len(sel)
    offA = np.concatenate([[0], np.cumsum(ns * ns)])
    offB = np.concatenate([[0], np.cumsum(ns * rs)])
    A0 = torch.empty(int(offA[-1]), dtype=torch.float64, device=dev)
    B0 = torch.empty(int(offB[-1]), dtype=torch.float64, device=dev)
    for i in range(cnt):
        n, r = int(ns[i]), int(rs[i])
        a = A0[offA[i]:offA[i + 1]].view(n, n).t()
        gi = int(sel[i])                                  # seeds follow the global system index
        if kinds[i] == 0:
            slt.generate(2, 10 * gi + 1, slt.colmajor(a))
        else:
            g = slt.colmajor(torch.empty(n, n, dtype=torch.float64, device=dev))
            slt.generate(3, 10 * gi + 1, g)
            a.copy_((g @ g.t()) / n + torch.eye(n, dtype=torch.float64, device=dev))
        slt.generate(2, 10 * gi + 2, slt.colmajor(B0[offB[i]:offB[i + 1]].view(r, n).t()))
    A = A0.clone()
    B = B0.clone()
    X = torch.zeros_like(B0)

    def views(Abuf, Bbuf):
        return [(int(kinds[i]), Abuf[offA[i]:offA[i + 1]].view(int(ns[i]), int(ns[i])).t(),
                 Bbuf[offB[i]:offB[i + 1]].view(int(rs[i]), int(ns[i])).t()) for i in range(cnt)]

    sysv = views(A, B)
    Xv = [X[offB[i]:offB[i + 1]].view(int(rs[i]), int(ns[i])).t() for i in range(cnt)]
    vb = slt.VBatch(sysv, X=Xv)
    flops = float(np.sum(np.where(kinds_all == 0, 2.0 * ns_all**3 / 3, ns_all**3 / 3.0) + 2.0 * ns_all * ns_all * rs_all))

    def berr_max(Xbuf):
        worst = 0.0
        for i in range(0, cnt, max(1, cnt // 2000)):      # every system up to 2000, else a stride sample
            k, a, b = int(kinds[i]), A0[offA[i]:offA[i + 1]].view(int(ns[i]), int(ns[i])).t(), \
                B0[offB[i]:offB[i + 1]].view(int(rs[i]), int(ns[i])).t()
            x = Xbuf[offB[i]:offB[i + 1]].view(int(rs[i]), int(ns[i])).t()
            if k == 1:
                a = torch.tril(a) + torch.tril(a, -1).t()
            rr = b - a @ x
            e = float(rr.abs().sum(0).max() / (a.shape[0] * a.abs().sum(0).max() * x.abs().sum(0).max()))
            worst = max(worst, e)
        return worst

    rec = {"config": 5, "workload": "%d systems, n log-uniform [32,1024], 1-8 RHS, half LU half SPD" % cnt,
           "flops": flops, "fp64_gb": 8.0 * float(offA[-1]) / 1e9}
    # batched FP64 (A, B restored outside the timing)
    ts = []
    for it in range(2):
        A.copy_(A0)
        B.copy_(B0)
        t, info = _event_time(torch, lambda: slt.solve_vbatched(vb))
        ts.append(t)
    def tmax(t):
        if ws > 1:
            tt = torch.tensor([t], device=dev)
            torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
            return float(tt.item())
        return t
    ts[-1] = tmax(ts[-1])
    rec["n_gpus"] = ws
    rec["batched_fp64_ms"] = ts[-1] * 1e3
    rec["batched_fp64_tflops"] = flops / ts[-1] / 1e12
    rec["batched_fp64_info_nonzero"] = int((info != 0).sum())
    rec["batched_fp64_berr_max"] = berr_max(B)
    # batched mixed
    A.copy_(A0)
    B.copy_(B0)
    ts = []
    for it in range(2):
        X.zero_()
        t, (info, iters) = _event_time(torch, lambda: slt.solve_mixed_vbatched(vb, slt.Options()))
        ts.append(t)
    ts[-1] = tmax(ts[-1])
    rec["batched_mixed_ms"] = ts[-1] * 1e3
    rec["batched_mixed_effective_tflops"] = flops / ts[-1] / 1e12
    rec["batched_mixed_phase_ms"] = {k: slt.timer("vbatched_mixed::" + k) * 1e3 for k in ("factor_lo", "refine", "fallback")}
    rec["batched_mixed_iter_hist"] = {str(int(v)): int(c) for v, c in zip(*np.unique(iters, return_counts=True))}
    rec["batched_mixed_berr_max"] = berr_max(X)
    if args.no_loop or ws > 1:
        if rank == 0:
            print(json.dumps(rec))
        if ws > 1:
            torch.distributed.destroy_process_group()
        return
    # per-system loop of the library's own gesv / posv (FP64), A, B restored first
    A.copy_(A0)
    B.copy_(B0)
    torch.cuda.synchronize()
    o = slt.Options(nb=256, ib=32)
    t0 = time.perf_counter()
    for k, a, b in sysv:
        if k == 0:
            slt.gesv(a, b, o)
        else:
            slt.posv(a, b, o)
    torch.cuda.synchronize()
    tl = time.perf_counter() - t0
    rec["loop_fp64_ms"] = tl * 1e3
    rec["loop_fp64_berr_max"] = berr_max(B)
    rec["speedup_batched_fp64_vs_loop"] = tl / (rec["batched_fp64_ms"] / 1e3)
    rec["speedup_batched_mixed_vs_loop"] = tl / (rec["batched_mixed_ms"] / 1e3)
    print(json.dumps(rec))


def measured_peaks(torch, dev):
    """FP64 and FP32 GEMM rates of cuBLAS on this GPU, measured in-run
    (n = 8192, best of 5, CUDA events): the denominators of the FP64- and
    FP32-pipe kernels' roofline fractions."""
    out = {}
    n = 8192
    torch.backends.cuda.matmul.allow_tf32 = False
    for name, dt in (("fp64", torch.float64), ("fp32", torch.float32)):
        a = torch.randn(n, n, dtype=dt, device=dev)
        b = torch.randn(n, n, dtype=dt, device=dev)
        c = a @ b
        best = None
        for _ in range(5):
            t, c = _event_time(torch, lambda: a @ b)
            best = t if best is None else min(best, t)
        out[name] = 2.0 * n**3 / best / 1e12
        del a, b, c
    torch.cuda.empty_cache()
    return out


# kernel classes of the library's launch profiler (include/slate_gb300.h)
PROF_CLASSES = ((1, "gemm64"), (2, "gemm32_simt"), (3, "gemm_tc"), (4, "panel"), (5, "trsm"), (6, "laswp"),
                (7, "fp64_residual"), (8, "chol_panel"), (9, "convert"), (10, "sweep"), (11, "digit_residual"))


def _roofline(dom, d, peaks, fp_peaks, steps, t_step):
    if dom == "gemm_tc":
        peak, bound, unit = peaks.get("bf16_tflops", 1900.0), "tensor", "TFLOP/s"
        src = "MEASURED_PEAKS.json bf16_tflops (burst), of measured"
        achieved = d["flops"] / d["seconds"] / 1e12
    elif dom in ("gemm32_simt",):
        peak, bound, unit = fp_peaks["fp32"], "fp32", "TFLOP/s"
        src = "cuBLAS SGEMM n=8192 measured in this run (FP32 pipe, no tensor cores), of measured"
        achieved = d["flops"] / d["seconds"] / 1e12
    elif dom in ("gemm64", "fp64_residual"):
        peak, bound, unit = fp_peaks["fp64"], "fp64", "TFLOP/s"
        src = "cuBLAS DGEMM n=8192 measured in this run (FP64 pipe), of measured"
        achieved = d["flops"] / d["seconds"] / 1e12
    else:
        peak, bound, unit = peaks.get("hbm_gbs", 6800.0), "hbm", "GB/s"
        src = "MEASURED_PEAKS.json hbm_gbs, of measured" if "hbm_gbs" in peaks else "fallback 6800 GB/s"
        achieved = d["bytes"] / d["seconds"] / 1e9
    traffic = None
    tp = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if os.path.exists(tp):
        t = json.load(open(tp)).get(dom)
        if t and d["launches"]:
            # the captured launch's DRAM bytes, scaled by algorithmic bytes per launch
            traffic = t["dram_bytes"] * (d["bytes"] / d["launches"]) / t["algorithmic_bytes"]
    return {"kernel": dom, "bound": bound, "achieved": achieved, "peak": peak, "unit": unit,
            "frac": achieved / peak, "traffic": traffic, "traffic_unit": "bytes per launch",
            "algorithmic_bytes_per_launch": d["bytes"] / d["launches"] if d["launches"] else None,
            "algorithmic_flops_per_launch": d["flops"] / d["launches"] if d["launches"] else None,
            "peak_source": src, "launches_per_step": d["launches"] / steps,
            "share_of_step": d["seconds"] / (t_step * steps)}


def main():
    args = parse()
    if args.impl == "reference":
        if args.config not in WORKLOADS:
            print(json.dumps({"impl": "reference", "unavailable": "the reference arm runs the headline configs 2 and 4"}))
            return
        return run_reference(args)
    import torch
    import slate_gb300 as slt
    if args.config not in WORKLOADS or (args.config == 4 and args.sweep):
        ws, rank, local = dist_env()
        if args.config == 5 and ws > 1:
            import torch.distributed as dist
            dist.init_process_group("nccl")
        elif ws > 1 and rank != 0:
            return                      # configs 1, 3, 4 --sweep: one replica on rank 0
        torch.cuda.set_device(local)
        dev = torch.device("cuda", local)
        if args.config == 1:
            return run_config1(args, slt, torch, dev)
        if args.config == 5:
            return run_config5(args, slt, torch, dev, ws, rank)
        return run_mixed_sweep(args, slt, torch, dev, args.config)
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    peaks = {}
    pp = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pp):
        peaks = json.load(open(pp))
    fp_peaks = measured_peaks(torch, dev)

    w = WORKLOADS[args.config]
    n, nrhs = args.n, args.nrhs
    A, B, Xt = make_headline_system(slt, torch, args, dev)
    X = slt.colmajor(torch.zeros(n, nrhs, dtype=torch.float64, device=dev))
    opts = slt.Options(nb=args.nb, ib=32, factor_precision=args.prec, residual_engine=args.residual_engine)
    solve = slt.posv_mixed_gmres if w["routine"] == "posv_mixed_gmres" else slt.posv_mixed

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()
            torch.cuda.synchronize()

    for _ in range(args.warmup):
        X.zero_()
        info, it, _ = solve(A, B, X, opts)
    barrier()
    clk = Clocks(local)
    clk.start()
    l0 = slt.lib().slt_launch_count()
    slt.lib().slt_profile_enable(1)
    stream = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    iters = []
    barrier()
    # BENCH_PROFILE_RANGE=1: only the timed steps inside the profiler range
    # (ncu --profile-from-start off captures exactly them)
    prange = os.environ.get("BENCH_PROFILE_RANGE") == "1"
    if prange:
        torch.cuda.profiler.start()
    e0.record(stream)
    for _ in range(args.steps):
        info, it, _ = solve(A, B, X, opts)
        iters.append(it)
    e1.record(stream)
    barrier()
    if prange:
        torch.cuda.profiler.stop()
    launches = slt.lib().slt_launch_count() - l0
    clocks = clk.stop()
    t_step = e0.elapsed_time(e1) / 1e3 / args.steps
    import ctypes
    prof = {}
    for kind, name in PROF_CLASSES:
        f, by, sec, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double(), ctypes.c_longlong()
        slt.lib().slt_profile_read(kind, ctypes.byref(f), ctypes.byref(by), ctypes.byref(sec), ctypes.byref(c))
        if c.value:
            prof[name] = {"flops": f.value, "bytes": by.value, "seconds": sec.value, "launches": c.value}
    slt.lib().slt_profile_enable(0)
    phases = {k: slt.timer(w["routine"] + k) for k in ("", "::potrf_lo", "::potrs_lo", "::retry_fp32")}
    berr = backward_error(torch, A, X, B)
    ferr = _rel_fwd(torch, X, Xt) if Xt is not None else None

    tmax = t_step
    if ws > 1:
        tt = torch.tensor([t_step], device=dev)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        tmax = float(tt.item())
    value = ws * posv_flops(n, nrhs) / tmax / 1e12

    # plain FP64 posv on the same system, once (A restored outside the timing)
    plain = None
    if not args.no_plain:
        A2 = A.clone()
        X2 = B.clone()
        torch.cuda.synchronize()
        p0 = torch.cuda.Event(enable_timing=True)
        p1 = torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        pinfo = slt.posv(slt.colmajor(A2), slt.colmajor(X2), slt.Options(nb=args.nb))
        p1.record(stream)
        torch.cuda.synchronize()
        tp = p0.elapsed_time(p1) / 1e3
        plain = {"value": posv_flops(n, nrhs) / tp / 1e12, "unit": "TFLOP/s", "ms": tp * 1e3,
                 "potrf_ms": slt.timer("posv::potrf") * 1e3,
                 "backward_error": backward_error(torch, A, X2, B), "info": pinfo}
        del A2, X2
        torch.cuda.empty_cache()

    # end to end through the LAPACK-compatible host entry point (pinned host buffers)
    e2e = None
    if not args.no_e2e:
        hA = torch.empty(n, n, dtype=torch.float64, pin_memory=True)
        hA.copy_(A.t())
        hB = torch.empty(nrhs, n, dtype=torch.float64, pin_memory=True)
        hB.copy_(B.t())
        hX = torch.zeros(nrhs, n, dtype=torch.float64, pin_memory=True)
        a_np, b_np, x_np = hA.numpy().T, hB.numpy().T, hX.numpy().T
        refine = "gmres" if w["routine"] == "posv_mixed_gmres" else "ir"
        ts = []
        ne = max(1, min(args.e2e_steps, args.steps))
        for i in range(1 + ne):
            t = time.perf_counter()
            ip = _dsposv(slt, a_np, b_np, x_np, args, refine)
            dt = time.perf_counter() - t
            if i >= 1:
                ts.append(dt)
        te = statistics.median(ts)
        e2e = {"value": ws * posv_flops(n, nrhs) / te / 1e12, "unit": "TFLOP/s",
               # the lower triangle of A in 512-column blocks (diagonal blocks whole), and B
               "h2d_bytes_per_step": lower_block_bytes(n, 512) + 8 * n * nrhs, "d2h_bytes_per_step": 8 * n * nrhs,
               "ms_per_step": te * 1e3, "steps": ne, "iter": ip,
               "entry_point": "slate_dsposv (LAPACK dsposv signature, host buffers), SLATE_LAPACK_REFINE=%s"
                              % refine}
        del hA, hB, hX

    if rank != 0:
        return
    dom = max(prof.items(), key=lambda kv: kv[1]["seconds"]) if prof else (None, None)
    roof = _roofline(dom[0], dom[1], peaks, fp_peaks, args.steps, t_step) if dom[0] else None
    cpu = cpu_baseline_sample(args) if (ws == 1 and rank == 0 and not args.no_cpu) else None
    line = {"metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": tmax * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config(args),
            "iter": iters[-1], "info": info, "backward_error": berr, "forward_error": ferr,
            "backward_error_bound_3n_eps": 3 * n * np.finfo(np.float64).eps,
            "phases_s": phases, "plain_fp64": plain,
            "speedup_vs_plain_fp64": (value / plain["value"]) if plain else None,
            "e2e": e2e, "gpu_launches": launches, "clocks": clocks, "roofline": roof,
            "measured_gemm_tflops": fp_peaks, "kernel_profile": prof, "cpu_baseline": cpu}
    print(json.dumps(line))
    if ws > 1:
        torch.distributed.destroy_process_group()


def lower_block_bytes(n, blk):
    """Bytes of A that slate_dsposv moves to the device: rows j0 .. n of every
    blk-column block (the referenced lower triangle, diagonal blocks whole)."""
    return sum(8 * (n - j0) * min(blk, n - j0) for j0 in range(0, n, blk))


def _dsposv(slt, a, b, x, args, refine):
    import ctypes
    c = ctypes.c_int
    n, nrhs = a.shape[0], b.shape[1]
    os.environ["SLATE_LAPACK_NB"] = str(args.nb)
    os.environ["SLATE_LAPACK_FACTOR_PRECISION"] = args.prec
    os.environ["SLATE_LAPACK_REFINE"] = refine
    it, info = c(0), c(0)
    slt.lib().slate_dsposv(ctypes.c_char_p(b"L"), ctypes.byref(c(n)), ctypes.byref(c(nrhs)),
                           a.ctypes.data_as(ctypes.c_void_p), ctypes.byref(c(n)),
                           b.ctypes.data_as(ctypes.c_void_p), ctypes.byref(c(n)),
                           x.ctypes.data_as(ctypes.c_void_p), ctypes.byref(c(n)), None, None,
                           ctypes.byref(it), ctypes.byref(info))
    if info.value != 0:
        raise RuntimeError("slate_dsposv info %d" % info.value)
    return it.value


if __name__ == "__main__":
    main()
