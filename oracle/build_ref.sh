#!/usr/bin/env bash
# Compile the reference's host-side query preprocessing (its own sources, read
# in place) with oracle/ref_plan_harness.cpp into oracle/_ref/ref_plan, and its
# data-graph loader with oracle/ref_load_harness.cpp into oracle/_ref/ref_load.
# TEST INFRASTRUCTURE ONLY: used to generate tests/golden/ref_plans.json and
# to time the reference's loader.
# Needs the reference tree (REF, default /root/reference); it is not on the
# GPU host, where this script is skipped.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${REF:-/root/reference}"
OUT="$HERE/_ref"
NVCC="${NVCC:-/usr/local/cuda/bin/nvcc}"
if [ ! -d "$REF" ]; then
  echo "reference tree not found at $REF; skipping" >&2
  exit 0
fi
mkdir -p "$OUT"
# The reference's globals.cuh declares extern __constant__ symbols that its
# kernels share across files, so it needs relocatable device code
# (CMakeLists.txt:57).  -DNDEBUG turns off its debug prints.
"$NVCC" -std=c++17 -O1 -DNDEBUG -rdc=true -gencode arch=compute_103a,code=sm_103a \
  -I"$REF" -I/usr/local/cuda/include -w \
  "$REF/io.cu" "$REF/cpuGraph.cpp" "$REF/gpuGraph.cpp" "$REF/decycle.cpp" "$REF/order.cpp" \
  "$REF/structure.cu" "$REF/filter.cu" "$REF/globals.cu" "$HERE/ref_plan_harness.cpp" \
  -o "$OUT/ref_plan"
echo "$OUT/ref_plan"
# The reference's data-graph loader alone, at -O3, for timing it beside the
# library's loader (oracle/ref_load_harness.cpp).
"$NVCC" -std=c++17 -O3 -Xcompiler -O3 -DNDEBUG -rdc=true -gencode arch=compute_103a,code=sm_103a \
  -I"$REF" -I/usr/local/cuda/include -w \
  "$REF/io.cu" "$REF/cpuGraph.cpp" "$REF/gpuGraph.cpp" "$REF/decycle.cpp" "$REF/order.cpp" \
  "$REF/structure.cu" "$REF/filter.cu" "$REF/globals.cu" "$HERE/ref_load_harness.cpp" \
  -o "$OUT/ref_load"
echo "$OUT/ref_load"
