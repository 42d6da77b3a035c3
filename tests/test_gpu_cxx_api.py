"""SLATE's C++ driver API (include/slate_gb300.hh) compiled against the
library and run on the GPU: gesv, getrs with the returned Pivots, posv,
posv_mixed, and exceptions on a grid other than 1 x 1."""
import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cxx_api(tmp_path, slt):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / "cxx_api_test")
    libdir = os.path.dirname(slt.LIB_PATH)
    subprocess.run([nvcc, "-std=c++17", "-O1", os.path.join(ROOT, "tests", "cxx", "cxx_api_test.cc"),
                    "-I" + os.path.join(ROOT, "include"), "-L" + libdir, "-lslate_gb300",
                    "-Xlinker", "-rpath=" + libdir, "-o", exe], check=True, capture_output=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip().endswith("OK"), (r.returncode, r.stdout, r.stderr)
