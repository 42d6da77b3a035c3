"""The C-ABI library builds, loads and exports every declared symbol (no GPU)."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if not f.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", f)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b((?:slt|slate)_\w+)\s*\(", text, re.M):
            names.add(m.group(1))
    return names


def test_header_declares_entry_points():
    names = declared_symbols()
    for must in ("slate_dgesv", "slate_dgesv_", "slate_dsgesv", "slate_dposv", "slate_dpotrf",
                 "slate_dgetrf", "slate_dgetrs", "slt_dgesv_device", "slt_dsgesv_device",
                 "slt_dsgesv_gmres_device", "slt_dsposv_device", "slt_dsposv_gmres_device",
                 "slt_dpotrf_device", "slt_dgetrf_device"):
        assert must in names


def test_library_exports_every_declared_symbol(slt):
    L = ctypes.CDLL(slt.LIB_PATH)
    missing = [n for n in sorted(declared_symbols()) if not hasattr(L, n)]
    assert not missing, missing


def test_host_only_calls(slt):
    L = slt.lib()
    assert b"sm_103a" in L.slt_version()
    assert L.slt_status_string(-2) == b"a bounded device wait timed out"
    o = slt._Options()
    L.slt_options_default(ctypes.byref(o))
    assert o.nb == 512 and o.max_iterations == 30 and o.use_fallback == 1


def test_options_mirror():
    import slate_gb300 as s
    o = s.Options(nb=256, factor_precision="bf16")._c()
    assert o.nb == 256 and o.factor_precision == s.PREC_BF16


def test_c_api_handles_host_only(slt):
    """SLATE's C API handles: options round trip, grid and tile checks."""
    L = slt.lib()
    vp, i64 = ctypes.c_void_p, ctypes.c_int64
    L.slate_Options_create.restype = vp
    o = L.slate_Options_create()
    L.slate_Options_set_BlockSize.argtypes = [vp, i64]
    L.slate_Options_get_BlockSize.argtypes = [vp, i64]
    L.slate_Options_get_BlockSize.restype = i64
    L.slate_Options_set_BlockSize(o, 256)
    assert L.slate_Options_get_BlockSize(o, 1) == 256
    L.slate_Options_get_BlockSize.argtypes = [vp, i64]
    assert L.slate_Options_get_BlockSize(None, 7) == 7
    L.slate_Options_set_Tolerance.argtypes = [vp, ctypes.c_double]
    L.slate_Options_get_Tolerance.argtypes = [vp, ctypes.c_double]
    L.slate_Options_get_Tolerance.restype = ctypes.c_double
    L.slate_Options_set_Tolerance(o, 1e-9)
    assert L.slate_Options_get_Tolerance(o, 0.0) == 1e-9
    L.slate_Options_destroy.argtypes = [vp]
    L.slate_Options_destroy(o)
    mk = L.slate_Matrix_create_fromScaLAPACK_r64
    mk.restype = vp
    mk.argtypes = [i64, i64, vp, i64, i64, i64, ctypes.c_int, ctypes.c_int, ctypes.c_ssize_t]
    import numpy as np
    a = np.zeros((8, 8), order="F")
    assert mk(8, 8, a.ctypes.data, 8, 4, 4, 2, 1, 0) is None        # 2 x 1 grid rejected
    assert mk(8, 8, a.ctypes.data, 8, 4, 2, 1, 1, 0) is None        # mb != nb rejected
    h = mk(8, 8, a.ctypes.data, 8, 4, 4, 1, 1, 0)
    assert h
    L.slate_Matrix_m_r64.argtypes = [vp]
    L.slate_Matrix_m_r64.restype = i64
    assert L.slate_Matrix_m_r64(h) == 8
    L.slate_Matrix_destroy_r64.argtypes = [vp]
    L.slate_Matrix_destroy_r64(h)


def test_device_scratch_sizes(slt):
    """Scratch the drivers allocate for one triangular sweep and one Cholesky
    panel launch (host-only size functions).  Sweep: 256 bytes of ticket,
    a mailbox of 16 right-hand sides x npad rows x two 8-byte words, then
    the 64 x 64 diagonal inverses and chain-step blocks W of every 64-row
    block, sized for double, then the row-major FP32 copy of the solution
    (npad x 16) and one done flag per block.  Panel: 512 bytes of counters, then one 64 x 64
    inverse per 64-column step (at most 16), sized for double."""
    L = slt.lib()
    L.slt_sweep_flags_bytes.restype = ctypes.c_size_t
    L.slt_sweep_flags_bytes.argtypes = [ctypes.c_int64]
    for n in (1, 63, 64, 65, 16384, 65537):
        nblk = -(-n // 64)
        npad = nblk * 64
        assert L.slt_sweep_flags_bytes(n) == (256 + 16 * npad * 2 * 8 + 2 * nblk * 64 * 64 * 8 +
                                              npad * 16 * 4 + nblk * 4)
    L.slt_chol_panel_ws_bytes.restype = ctypes.c_size_t
    L.slt_chol_panel_ws_bytes.argtypes = []
    assert L.slt_chol_panel_ws_bytes() == 512 + 16 * 64 * 64 * 8


def test_noalloc_segment_plan_fits_the_scratch(slt):
    """The allocation-free residual's column-segment plan (host only): for
    orders near the 2,097,152-double scratch with 16 right-hand sides the
    plan lowers the segment count until nseg * n * nc fits, the segments
    cover every 64-column tile, and one segment too large is refused."""
    L = slt.lib()
    f = L.slt_noalloc_segment_plan
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int64, ctypes.c_int64, ctypes.c_uint64, ctypes.POINTER(ctypes.c_int64),
                  ctypes.POINTER(ctypes.c_int64)]
    ws = 2097152
    lowered = 0
    for n in (1, 64, 3000, 40000, 60000, 65600, 70000, 100000, 131072):
        for nc in (1, 4, 16):
            nseg, tps = ctypes.c_int64(), ctypes.c_int64()
            rc = f(n, nc, ws, ctypes.byref(nseg), ctypes.byref(tps))
            if n * nc > ws:
                assert rc != 0, (n, nc)
                continue
            assert rc == 0, (n, nc, rc)
            ktiles = -(-n // 64)
            assert nseg.value >= 1 and tps.value >= 1
            assert nseg.value * n * nc <= ws, (n, nc, nseg.value)
            assert (nseg.value - 1) * tps.value < ktiles <= nseg.value * tps.value, (n, nc, nseg.value, tps.value)
            unconstrained = min(ktiles, -(-152 * 8 // -(-n // 64)))
            lowered += nseg.value < unconstrained
    assert lowered > 0                        # the lowering branch ran
