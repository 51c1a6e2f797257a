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
# The reference's SSSP callbacks on this library's engine (ref_engine_sssp.cu):
# the four process_edges callbacks of toolkits/sssp.cpp, each lambda made a
# by-value __device__ lambda, compiled against gemini/engine.cuh.  Needs nvcc
# and the library (built first by __graft_entry__.build()).
REPO="$(cd "$HERE/.." && pwd)"
LIB="$REPO/geminigraph_gb300/libgemini_gb300.so"
NVCC="${NVCC:-/usr/local/cuda/bin/nvcc}"
INC="$SRC/sssp_callbacks.inc"
awk '/graph->process_edges<VertexId,Weight>\(/ {on = 1; next} on && /^[[:space:]]*active_in[[:space:]]*$/ {exit} on {print}' \
  "$SRC/toolkits/sssp.cpp" | sed 's/\[&\](/[=] __device__ (/g' > "$INC.tmp"
if ! cmp -s "$INC.tmp" "$INC"; then mv "$INC.tmp" "$INC"; else rm -f "$INC.tmp"; fi
if [ -x "$NVCC" ] && [ -f "$LIB" ] && [ -s "$INC" ]; then
  if ! [ "$BIN/ref_engine_sssp" -nt "$HERE/ref_engine_sssp.cu" ] || ! [ "$BIN/ref_engine_sssp" -nt "$INC" ] ||
     ! [ "$BIN/ref_engine_sssp" -nt "$REPO/geminigraph_gb300/cpp/gemini/engine.cuh" ] ||
     ! [ "$BIN/ref_engine_sssp" -nt "$LIB" ]; then
    "$NVCC" -gencode arch=compute_103a,code=sm_103a -O3 -std=c++17 --extended-lambda \
      -I"$REPO/include" -I"$REPO/geminigraph_gb300/cpp" -I"$SRC" "$HERE/ref_engine_sssp.cu" \
      -o "$BIN/ref_engine_sssp" -L"$REPO/geminigraph_gb300" -lgemini_gb300 \
      -Xlinker -rpath,'$ORIGIN/../../../geminigraph_gb300'
  fi
fi
echo "build_ref: toolkits in $BIN"
