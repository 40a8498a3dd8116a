#!/bin/bash
# Compiles MDcraft's own C++ tests (test/cxx/{domain,neibs,solver}/*.cxx of a
# reference checkout, unmodified, with test/cxx/support/md_test_utils.h)
# against this library's C++ drop-in headers and the GoogleTest stand-in
# beside this script, links them with libmdg, and with --run runs them.
#
#   reference_tests.sh [--run] [REFERENCE_DIR] [OUT_DIR]
#
# REFERENCE_DIR defaults to /root/reference; the tests read their fixtures
# (test/cxx/LMP_BALL_130k_Ar, test/python/solver/Al2009.eam.alloy) under it.
# Exit status 77: no reference test sources there (nothing was built).
set -e
RUN=0
if [ "$1" = "--run" ]; then RUN=1; shift; fi
REF=${1:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
ROOT=$(cd "$HERE/../../.." && pwd)
OUT=${2:-$ROOT/mdcraft_gb300/_build/reference_tests}
TESTS="domain/test_domain neibs/test_grid neibs/test_verlet_list solver/test_ljs_cut solver/test_argon_ball_md solver/test_aluminum_bulk_eam"
for t in $TESTS; do
  [ -f "$REF/test/cxx/$t.cxx" ] || { echo "no reference test sources under $REF"; exit 77; }
done
[ -f "$REF/test/cxx/support/md_test_utils.h" ] || { echo "no $REF/test/cxx/support/md_test_utils.h"; exit 77; }
python -c "import sys; sys.path.insert(0, '$ROOT'); from mdcraft_gb300 import build as B; B.build()"
CUDA=$(dirname "$(dirname "$(command -v nvcc || echo /usr/local/cuda/bin/nvcc)")")
# the support header is included as <test/cxx/support/md_test_utils.h>: an
# include root holding only that folder, so no other reference header can
# stand in for a drop-in one
mkdir -p "$OUT/inc/test/cxx"
ln -sfn "$REF/test/cxx/support" "$OUT/inc/test/cxx/support"
SRCS=""
for t in $TESTS; do SRCS="$SRCS $REF/test/cxx/$t.cxx"; done
g++ -std=c++17 -O2 -I "$HERE" -I "$ROOT/mdcraft_gb300/cxx/include" -I "$ROOT/include" -I "$CUDA/include" \
    -I "$OUT/inc" -DMDCRAFT_SOURCE_DIR="\"$REF\"" $SRCS "$HERE/gtest/gtest_main.cpp" \
    -L "$ROOT/mdcraft_gb300/_build" -lmdg -L "$CUDA/lib64" -lcudart -Wl,-rpath,"$ROOT/mdcraft_gb300/_build" \
    -o "$OUT/run_tests"
echo "built $OUT/run_tests"
if [ $RUN = 1 ]; then "$OUT/run_tests"; fi
