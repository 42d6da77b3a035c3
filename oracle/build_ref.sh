#!/bin/bash
# Compile SLATE's own Philox generator (matgen/random.cc) from the SLATE source
# tree into oracle/_ref/libref_random.so.  SLATE's build system is not used:
# random.cc needs only two BLAS++ type utilities, supplied by oracle/refshim/.
# Skips quietly when the SLATE sources are not present (e.g. on a GPU host).
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
SRC="${SLATE_SRC:-/root/reference}"
if [ ! -f "$SRC/matgen/random.cc" ]; then
    echo "build_ref: SLATE sources not found at $SRC; skipping"
    exit 0
fi
mkdir -p "$HERE/_ref"
g++ -O2 -std=c++17 -fPIC -shared -I"$HERE/refshim" -I"$SRC/matgen" \
    "$SRC/matgen/random.cc" "$HERE/ref_random_capi.cc" -o "$HERE/_ref/libref_random.so"
echo "build_ref: built $HERE/_ref/libref_random.so"
