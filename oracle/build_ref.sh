#!/usr/bin/env bash
# Builds the reference GraphPi library from its own sources, where they lie
# under the read-only reference checkout, into oracle/_ref/libgraphpi_ref.so
# (git-ignored).  Test infrastructure only: it pins the CPU oracle against the
# reference itself.  MPI is absent here, so oracle/mpi_stub/mpi.h stands in
# at compile time; the single-node path never calls MPI.
#
# usage: oracle/build_ref.sh [REFERENCE_ROOT]   (default /root/reference)
set -euo pipefail
REF="${1:-/root/reference}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -d "$REF/src" ]; then
  echo "reference sources not found at $REF; skipping oracle/_ref" >&2
  exit 0
fi
mkdir -p "$OUT"
SRCS="graph.cpp dataloader.cpp pattern.cpp prefix.cpp schedule.cpp vertex_set.cpp motif_generator.cpp graphmpi.cpp common.cpp disjoint_set_union.cpp"
OBJS=""
PIDS=""
for s in $SRCS; do
  o="$OUT/${s%.cpp}.o"
  g++ -std=c++11 -O3 -fopenmp -fPIC -w -I"$HERE/mpi_stub" -I"$REF/include" -c "$REF/src/$s" -o "$o" &
  PIDS="$PIDS $!"
  OBJS="$OBJS $o"
done
g++ -std=c++11 -O3 -fopenmp -fPIC -w -I"$HERE/mpi_stub" -I"$REF/include" -c "$HERE/ref_shim.cpp" -o "$OUT/ref_shim.o" &
PIDS="$PIDS $!"
for p in $PIDS; do wait "$p"; done
g++ -shared -fopenmp -o "$OUT/libgraphpi_ref.so" $OBJS "$OUT/ref_shim.o"
rm -f $OBJS "$OUT/ref_shim.o"
echo "built $OUT/libgraphpi_ref.so"
