#!/bin/sh
# Builds the reference's own CPU MDSystem (vlvovch/lennard-jones-cuda,
# src/library/MDSystem.cpp + splinefunction.cpp, read where they lie) plus the
# C shim oracle/ref_shim.cpp into oracle/_ref/libmdsystem_ref.so.
# -O2 is the reference's RelWithDebInfo level; -ffp-contract=off keeps its
# float/double rounding identical on x86-64 and aarch64.  Test infrastructure
# only: the output is git-ignored and never linked by the product.
set -e
REF=${LJ_REFERENCE_DIR:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -f "$REF/src/library/MDSystem.cpp" ]; then
  echo "reference sources not found under $REF; skipping oracle/_ref" >&2
  exit 0
fi
mkdir -p "$OUT"
g++ -std=c++11 -O2 -g -fPIC -shared -ffp-contract=off -w \
  -I "$REF/src/library" -I "$REF/thirdparty" \
  "$REF/src/library/MDSystem.cpp" "$REF/src/library/splinefunction.cpp" "$HERE/ref_shim.cpp" \
  -o "$OUT/libmdsystem_ref.so"
echo "built $OUT/libmdsystem_ref.so"
