#!/bin/sh
# Compiles the reference's own pair-potential headers (potential/*.h) and the
# Octic / Rect / Mollifier headers
# (header-only, no external dependencies) into oracle/_ref/libref_kernels.so.
# Only possible where the reference tree exists; outputs go to oracle/_ref only.
# -ffp-contract=off matches the oracle's evaluation (the reference's own build
# uses -O3 -march=native, which may contract a*b+c into FMA on FMA hosts).
set -e
REF=${PYGLASSTOOLS_REF:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
if [ ! -f "$REF/pyglasstools/potential/Polydisperse12.h" ]; then
  echo "reference tree not found at $REF; skipping oracle/_ref" >&2
  exit 0
fi
mkdir -p "$HERE/_ref"
CG="$REF/pyglasstools/irvingkirkwood/cgfunc"
${CXX:-g++} -O2 -fPIC -shared -ffp-contract=off -std=c++14 \
  -I "$REF/pyglasstools/potential" -I "$CG" \
  -o "$HERE/_ref/libref_kernels.so" "$HERE/ref_kernels.cpp"
echo "built $HERE/_ref/libref_kernels.so"
