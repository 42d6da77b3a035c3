"""Build libslate_gb300.so in-tree for sm_103a (nvcc, parallel compile, no cmake).

    python -m slate_gb300.build [--verbose] [--ptxas-info]
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libslate_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
          "-I" + CSRC, "-I" + os.path.join(ROOT, "include")]


def nvcc():
    for p in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if p and os.path.exists(p):
            return p
    raise RuntimeError("nvcc not found")


def sources():
    out = []
    for f in sorted(os.listdir(CSRC)):
        if f.endswith(".cu") or f.endswith(".cc"):
            out.append(os.path.join(CSRC, f))
    return out


def _compile(src, verbose=False, ptxas_info=False):
    obj = os.path.join(OBJ, os.path.basename(src) + ".o")
    cmd = [nvcc(), "-c", src, "-o", obj] + COMMON
    if src.endswith(".cu"):
        cmd += ARCH
        if ptxas_info:
            cmd += ["-Xptxas", "-v"]
    else:
        cmd += ["-x", "c++"]
    # rebuild only when stale
    deps = [src] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    deps.append(os.path.join(ROOT, "include", "slate_gb300.h"))
    if (not ptxas_info and os.path.exists(obj)
            and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps)):
        return obj, ""
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return obj, (r.stdout + r.stderr) if (verbose or ptxas_info) else ""


def build(verbose=False, ptxas_info=False):
    os.makedirs(OBJ, exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose, ptxas_info), srcs))
    for _, log in results:
        if log:
            sys.stdout.write(log)
    objs = [o for o, _ in results]
    newest = max(os.path.getmtime(o) for o in objs)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        cmd = [nvcc(), "-shared", "-o", LIB] + objs + ARCH + ["-Xcompiler", "-fPIC", "-lcudart_static",
                                                               "-lrt", "-lpthread", "-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return LIB


if __name__ == "__main__":
    build(verbose="--verbose" in sys.argv, ptxas_info="--ptxas-info" in sys.argv)
    print(LIB)
