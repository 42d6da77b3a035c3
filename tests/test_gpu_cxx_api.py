"""SLATE's C++ driver API (include/slate_gb300.hh) compiled against the
library and run on the GPU: gesv, getrs with the returned Pivots, posv,
posv_mixed, exceptions on a grid other than 1 x 1 (cxx_api_test.cc); the
tile storage model -- host-origin fromLAPACK, insertLocalTiles on the host
and the device, user-owned tiles, MOSI states, complex and single precision,
Upper Hermitian storage (tile_matrix_test.cc)."""
import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("src", ["cxx_api_test.cc", "tile_matrix_test.cc"])
def test_cxx_api(tmp_path, slt, src):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / src.replace(".cc", ""))
    libdir = os.path.dirname(slt.LIB_PATH)
    subprocess.run([nvcc, "-std=c++17", "-O1", os.path.join(ROOT, "tests", "cxx", src),
                    "-I" + os.path.join(ROOT, "include"), "-L" + libdir, "-lslate_gb300",
                    "-Xlinker", "-rpath=" + libdir, "-o", exe], check=True, capture_output=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip().endswith("OK"), (r.returncode, r.stdout, r.stderr)
