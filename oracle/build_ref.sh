#!/bin/sh
# Builds the unmodified reference Multistep code (HPCGraphAnalysis/Connectivity
# multistep/) into oracle/_ref/ through oracle/ref_harness.cpp.
#
# Test infrastructure only.  The sources are read from $REF_DIR when it is
# set, else from baseline/_ref/multistep, the git-ignored reference install
# that oracle/install_ref.sh makes (an unmodified copy of the reference's
# multistep/ directory, which travels with the working tree to machines that
# do not hold the reference).  Nothing is written outside oracle/_ref/.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
ROOT=$(dirname "$HERE")
REF_DIR=${REF_DIR:-$ROOT/baseline/_ref/multistep}
OUT="$HERE/_ref"
if [ ! -f "$REF_DIR/scc_main.cpp" ]; then
  echo "reference sources not found at $REF_DIR; oracle/_ref not built" >&2
  exit 0
fi
mkdir -p "$OUT"
CXX=${CXX:-g++}
FLAGS="-O3 -fopenmp -w"
$CXX $FLAGS -DREF_SRC_SCC="\"$REF_DIR/scc_main.cpp\"" "$HERE/ref_harness.cpp" -o "$OUT/ref_scc" &
$CXX $FLAGS -DREF_CC -DREF_SRC_CC="\"$REF_DIR/cc_main.cpp\"" "$HERE/ref_harness.cpp" -o "$OUT/ref_cc" &
wait
echo "built $OUT/ref_scc $OUT/ref_cc"
