#!/bin/sh
# Builds the reference's own CPU code from its sources, read where they lie in
# a vlvovch/lennard-jones-cuda checkout given as the first argument (or in
# LJ_REFERENCE_DIR):
#   * src/library/MDSystem.cpp + splinefunction.cpp plus the C shim
#     oracle/ref_shim.cpp -> oracle/_ref/libmdsystem_ref.so;
#   * oracle/ref_stats_driver.cpp over the header-only statistics
#     (src/extra/sample-moments/NumberStatistics.h,
#     src/tasks/auxiliary/time-average-aux.h) -> oracle/_ref/ref_stats.
# -O2 is the reference's RelWithDebInfo level; -ffp-contract=off keeps its
# float/double rounding identical on x86-64 and aarch64.  Test infrastructure
# only: the outputs are git-ignored and never linked by the product.
set -e
REF=${1:-$LJ_REFERENCE_DIR}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ -z "$REF" ] || [ ! -f "$REF/src/library/MDSystem.cpp" ]; then
  echo "reference sources not given or not found (${REF:-no directory}); skipping oracle/_ref" >&2
  exit 0
fi
mkdir -p "$OUT"
g++ -std=c++11 -O2 -g -fPIC -shared -ffp-contract=off -w \
  -I "$REF/src/library" -I "$REF/thirdparty" \
  "$REF/src/library/MDSystem.cpp" "$REF/src/library/splinefunction.cpp" "$HERE/ref_shim.cpp" \
  -o "$OUT/libmdsystem_ref.so"
echo "built $OUT/libmdsystem_ref.so"
g++ -std=c++11 -O2 -ffp-contract=off -w \
  -I "$REF/src/library" -I "$REF/thirdparty" -I "$REF/src/extra/sample-moments" -I "$REF/src/tasks/auxiliary" \
  "$HERE/ref_stats_driver.cpp" -o "$OUT/ref_stats"
echo "built $OUT/ref_stats"
