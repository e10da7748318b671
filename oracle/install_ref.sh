#!/bin/sh
# Installs the reference Multistep sources for the checker:
#
#     sh oracle/install_ref.sh <reference tree>
#
# copies <reference tree>/multistep/ unmodified into baseline/_ref/multistep/
# (git-ignored: it is the reference, not this project's source).  The copy
# travels with the working tree, so oracle/build_ref.sh can compile the
# reference on a machine that does not hold the reference tree (the GPU
# host's own cores time it there).  Test infrastructure only.
set -e
if [ $# -ne 1 ] || [ ! -f "$1/multistep/scc_main.cpp" ]; then
  echo "usage: $0 <reference tree containing multistep/scc_main.cpp>" >&2
  exit 2
fi
HERE=$(cd "$(dirname "$0")" && pwd)
ROOT=$(dirname "$HERE")
DEST="$ROOT/baseline/_ref/multistep"
mkdir -p "$DEST"
cp "$1"/multistep/*.cpp "$1"/multistep/README "$DEST"/
echo "installed $DEST"
