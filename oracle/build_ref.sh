#!/bin/sh
# Builds oracle/_ref/libxyst_ref.so from the reference's own, unmodified
# physics sources where they lie, plus the stub headers in oracle/ref_stubs and
# the shim oracle/ref_driver.cpp.  Test infrastructure only: the result pins the
# C++ restatement in oracle/xg_oracle.cpp.  Outputs go to oracle/_ref/ only.
#   usage: oracle/build_ref.sh [reference-root]
#   (default: $XYST_REFERENCE, else a checkout named "reference" beside this repository)
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${1:-${XYST_REFERENCE:-$HERE/../../reference}}
OUT="$HERE/_ref"
if [ ! -d "$REF/src/Physics" ]; then
  echo "reference sources not found at $REF; skipping" >&2
  exit 3
fi
mkdir -p "$OUT"
S="$REF/src"
INC="-I$HERE/ref_stubs -I$S/Base -I$S/Physics -I$S/Control -I$S/Mesh -I$S/LinearSolver -I$S -I$S/Main -I$S/brigand -I$S/Inciter"
SRCS="$S/Physics/Riemann.cpp $S/Physics/Kozak.cpp $S/Physics/Chorin.cpp $S/Physics/Problems.cpp $S/Physics/Box.cpp $S/Physics/BC.cpp $S/LinearSolver/CSR.cpp $S/Mesh/DerivedData.cpp $S/Mesh/Reorder.cpp $S/Base/Exception.cpp $HERE/ref_driver.cpp"
pids=""
objs=""
for f in $SRCS; do
  o="$OUT/$(basename "$f" .cpp).o"
  objs="$objs $o"
  g++ -std=c++17 -O2 -ffp-contract=off -fPIC -w $INC -c "$f" -o "$o" &
  pids="$pids $!"
done
for p in $pids; do wait "$p"; done
g++ -shared -o "$OUT/libxyst_ref.so" $objs
rm -f $objs
echo "built $OUT/libxyst_ref.so"
