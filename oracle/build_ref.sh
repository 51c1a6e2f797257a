#!/usr/bin/env bash
# Builds the Gemini reference toolkits (bfs, cc, pagerank, sssp, bc) from the
# reference's own sources, for use as test infrastructure and as the CPU
# baseline.  Outputs go only to oracle/_ref/ (git-ignored).
#
# Usage: build_ref.sh [<reference checkout>]  (or GG_REFERENCE_DIR=<dir>).
# Step 1 (only where a reference checkout is given): stage the reference's
#   core/*.hpp and toolkits/*.cpp into oracle/_ref/src/, applying two patches
#   to the staged copy of core/graph.hpp:
#     a. core/graph.hpp:240  `T * dealloc_vertex_array` -> `void ...`.  The
#        function falls off its end; GCC >= 8 at -O3 treats that as
#        unreachable and every toolkit crashes right after compute().
#     b. core/graph.hpp:1591,1713,1807 `pause` -> `yield` on aarch64 hosts
#        (x86 spin hint; does not assemble on Arm).
# Step 2 (wherever oracle/_ref/src exists): compile each toolkit with g++
#   against the single-rank MPI and one-node libnuma stand-ins in
#   oracle/shim/, exactly as the reference Makefile would with mpicxx
#   (-O3 -std=c++11 -fopenmp -march=native), into oracle/_ref/bin/.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${1:-${GG_REFERENCE_DIR:-}}"
OUT="$HERE/_ref"
SRC="$OUT/src"
BIN="$OUT/bin"

if [ -n "$REF" ] && [ -f "$REF/core/graph.hpp" ]; then
  mkdir -p "$SRC/core" "$SRC/toolkits"
  cp "$REF"/core/*.hpp "$SRC/core/"
  cp "$REF"/toolkits/*.cpp "$SRC/toolkits/"
  sed -i 's/^  T \* dealloc_vertex_array(T \* array) {/  void dealloc_vertex_array(T * array) {/' "$SRC/core/graph.hpp"
  grep -q 'void dealloc_vertex_array' "$SRC/core/graph.hpp"
fi

if [ ! -f "$SRC/core/graph.hpp" ]; then
  echo "build_ref: no reference sources staged under $SRC; skipping" >&2
  exit 0
fi

case "$(uname -m)" in
  aarch64|arm64) sed -i 's/__asm volatile ("pause" ::: "memory");/__asm volatile ("yield" ::: "memory");/' "$SRC/core/graph.hpp" ;;
esac

mkdir -p "$BIN"
CXX="${CXX:-g++}"
pids=()
for app in bfs cc pagerank sssp bc; do
  if [ "$BIN/$app" -nt "$SRC/toolkits/$app.cpp" ] && [ "$BIN/$app" -nt "$SRC/core/graph.hpp" ]; then
    continue
  fi
  "$CXX" -O3 -std=c++11 -g -fopenmp -march=native -w \
    -I"$HERE/shim" -I"$SRC" -o "$BIN/$app" "$SRC/toolkits/$app.cpp" -lpthread &
  pids+=($!)
done
# drivers: the same toolkits' compute() over several roots on one loaded graph
for app in bfs cc pagerank sssp bc; do
  APP=$(echo "$app" | tr a-z A-Z)
  if [ "$BIN/ref_$app" -nt "$HERE/ref_driver.cpp" ] && [ "$BIN/ref_$app" -nt "$SRC/core/graph.hpp" ] &&
     [ "$BIN/ref_$app" -nt "$HERE/shim/numa.h" ] && [ "$BIN/ref_$app" -nt "$HERE/shim/mpi.h" ]; then
    continue
  fi
  "$CXX" -O3 -std=c++11 -g -fopenmp -march=native -w -DGG_APP_$APP \
    -I"$HERE/shim" -I"$SRC" -o "$BIN/ref_$app" "$HERE/ref_driver.cpp" -lpthread &
  pids+=($!)
done
for p in "${pids[@]}"; do wait "$p"; done
echo "build_ref: toolkits in $BIN"
