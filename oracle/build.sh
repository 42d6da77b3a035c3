#!/bin/bash
# Build the CPU oracle (test infrastructure) into oracle/liboracle.so.
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
g++ -O3 -std=c++17 -fPIC -shared -fopenmp "$HERE/oracle.cc" -o "$HERE/liboracle.so"
echo "build: built $HERE/liboracle.so"
