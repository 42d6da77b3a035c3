#!/bin/bash
# Compile two pieces of SLATE from the SLATE source tree into oracle/_ref/,
# without SLATE's build system:
#  * libref_random.so: its Philox generator (matgen/random.cc), which needs
#    only two BLAS++ type utilities, supplied by oracle/refshim/;
#  * libref_getrf.so: its tile LU panel (src/internal/Tile_getrf.hh) with
#    SLATE's own ThreadBarrier and cabs1 (include/slate/internal/util.hh),
#    against the stand-ins of oracle/refshim_getrf/ for BLAS++, LAPACK++,
#    MPI (one process) and the Tile class, driven by oracle/ref_getrf_capi.cc.
# The SLATE source tree is the first argument or $SLATE_SRC; there is no
# default.  Skips quietly when neither names a tree holding matgen/random.cc
# (e.g. on a GPU host, which only uses the prebuilt files).
#
#     bash oracle/build_ref.sh <SLATE_SOURCE_DIR>
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
SRC="${1:-${SLATE_SRC:-}}"
if [ -z "$SRC" ] || [ ! -f "$SRC/matgen/random.cc" ]; then
    echo "build_ref: no SLATE source tree given (argument or SLATE_SRC) or matgen/random.cc missing; skipping"
    exit 0
fi
mkdir -p "$HERE/_ref"
g++ -O2 -std=c++17 -fPIC -shared -I"$HERE/refshim" -I"$SRC/matgen" \
    "$SRC/matgen/random.cc" "$HERE/ref_random_capi.cc" -o "$HERE/_ref/libref_random.so"
echo "build_ref: built $HERE/_ref/libref_random.so"
if [ -f "$SRC/src/internal/Tile_getrf.hh" ] && [ -f "$SRC/include/slate/internal/util.hh" ]; then
    g++ -O2 -std=c++17 -fPIC -shared -pthread -I"$HERE/refshim_getrf" -I"$SRC/src" -I"$SRC/include" \
        "$HERE/ref_getrf_capi.cc" -o "$HERE/_ref/libref_getrf.so"
    echo "build_ref: built $HERE/_ref/libref_getrf.so"
fi
