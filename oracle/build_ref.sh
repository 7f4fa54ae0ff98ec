#!/bin/sh
# Compiles the reference's own CPU solvers (unmodified headers, read in place
# from the reference checkout) into oracle/_ref/libref_dpbf.so, together with
# the Boost.Heap stand-in under oracle/ref/shim. Test infrastructure only.
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]
#   (default: $GST_REFERENCE_ROOT, else the "reference" directory beside
#   this repository's checkout)
set -eu
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${1:-${GST_REFERENCE_ROOT:-$HERE/../../reference}}
if [ ! -f "$REF/rucgraph/graph_v_of_v_idealID_DPBF_only_ec.h" ]; then
  echo "reference sources not found under $REF" >&2
  exit 3
fi
mkdir -p "$HERE/_ref"
g++ -std=c++17 -O2 -w -shared -fPIC \
  -I "$HERE/ref/shim" -I "$REF/rucgraph" \
  "$HERE/ref/ref_dpbf.cpp" -o "$HERE/_ref/libref_dpbf.so"
echo "built $HERE/_ref/libref_dpbf.so"
