#!/usr/bin/env bash
# Build the reference ClusterSM from its own sources, into oracle/_ref/.
# TEST INFRASTRUCTURE ONLY: the programs built here generate golden fixtures
# (ref_plan), time the reference's loader (ref_load) and run the reference's
# GPU filter and join as the parity anchor and timed baseline (ClusterSM,
# ref_match).  Nothing in the library links or calls them.
#
#   bash oracle/build_ref.sh [stage] [host] [gpu]
#   (default: all three from a reference checkout, gpu from the staged copy;
#   programs newer than their sources are not rebuilt)
#
#   stage  copy the reference's source files into oracle/_ref/src/ so that a
#          machine without the reference checkout (the GPU host) can build
#          them; oracle/_ref/ is git-ignored, so the copy is never committed
#   host   ref_plan, ref_load: the reference's host-side query preprocessing
#          and loader with small drivers; they call no CUDA API
#   gpu    ClusterSM: the unmodified reference binary (main.cu + its sources);
#          ref_match: the reference's filter and join over many queries
#          (oracle/ref_match_harness.cpp)
#
# The sources are read from $REF if set, else from a reference checkout next
# to this repository (../reference), else from the staged copy.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
SRC_COPY="$OUT/src"
NVCC="${NVCC:-/usr/local/cuda/bin/nvcc}"
FILES="CLI11.hpp cpuGraph.cpp cpuGraph.h cuda_helpers.h decycle.cpp decycle.h defs.h filter.cu filter.cuh
globals.cu globals.cuh gpuGraph.cpp gpuGraph.h io.cu io.cuh join.cu join.cuh main.cu memManag.cuh order.cpp
order.h structure.cu structure.cuh"

if [ -n "${REF:-}" ]; then
  :
elif [ -f "$HERE/../../reference/filter.cu" ]; then
  REF="$(cd "$HERE/../../reference" && pwd)"
elif [ -f "$SRC_COPY/filter.cu" ]; then
  REF="$SRC_COPY"
else
  echo "reference sources not found (set REF); skipping" >&2
  exit 0
fi

targets="$*"
if [ -z "$targets" ]; then
  if [ "$REF" = "$SRC_COPY" ]; then targets="gpu"; else targets="stage host gpu"; fi
fi
mkdir -p "$OUT"

# true when $1 is missing or older than any of the other arguments
stale() {
  local out="$1"
  shift
  [ -e "$out" ] || return 0
  for f in "$@"; do [ "$f" -nt "$out" ] && return 0; done
  return 1
}
SOURCES=""
for f in $FILES; do SOURCES="$SOURCES $REF/$f"; done

for t in $targets; do
  case "$t" in
    stage)
      if [ "$REF" != "$SRC_COPY" ]; then
        mkdir -p "$SRC_COPY"
        for f in $FILES; do install -m 0644 "$REF/$f" "$SRC_COPY/$f"; done
        echo "$SRC_COPY"
      fi
      ;;
    host)
      stale "$OUT/ref_load" $SOURCES "$HERE/ref_plan_harness.cpp" "$HERE/ref_load_harness.cpp" || continue
      # The reference's globals.cuh declares extern __constant__ symbols that
      # its kernels share across files, so it needs relocatable device code
      # (CMakeLists.txt:57).  -DNDEBUG turns off its debug prints.
      "$NVCC" -std=c++17 -O1 -DNDEBUG -rdc=true -gencode arch=compute_103a,code=sm_103a \
        -I"$REF" -I/usr/local/cuda/include -w \
        "$REF/io.cu" "$REF/cpuGraph.cpp" "$REF/gpuGraph.cpp" "$REF/decycle.cpp" "$REF/order.cpp" \
        "$REF/structure.cu" "$REF/filter.cu" "$REF/globals.cu" "$HERE/ref_plan_harness.cpp" \
        -o "$OUT/ref_plan"
      echo "$OUT/ref_plan"
      # The loader alone, at -O3, for timing it beside the library's loader.
      "$NVCC" -std=c++17 -O3 -Xcompiler -O3 -DNDEBUG -rdc=true -gencode arch=compute_103a,code=sm_103a \
        -I"$REF" -I/usr/local/cuda/include -w \
        "$REF/io.cu" "$REF/cpuGraph.cpp" "$REF/gpuGraph.cpp" "$REF/decycle.cpp" "$REF/order.cpp" \
        "$REF/structure.cu" "$REF/filter.cu" "$REF/globals.cu" "$HERE/ref_load_harness.cpp" \
        -o "$OUT/ref_load"
      echo "$OUT/ref_load"
      ;;
    gpu)
      stale "$OUT/ref_match" $SOURCES "$HERE/ref_match_harness.cpp" || continue
      # Optimised build (-O3, -DNDEBUG) for sm_103a with relocatable device
      # code, as CMakeLists.txt:54-57 links it; the shipped CMakeLists targets
      # sm_86 and a Debug host build.
      OBJ="$OUT/obj"
      mkdir -p "$OBJ"
      FLAGS="-std=c++17 -O3 -Xcompiler -O3 -DNDEBUG -rdc=true -lineinfo -gencode arch=compute_103a,code=sm_103a -I$REF -I/usr/local/cuda/include -w"
      pids=()
      for f in io.cu cpuGraph.cpp gpuGraph.cpp decycle.cpp order.cpp structure.cu filter.cu globals.cu join.cu main.cu; do
        "$NVCC" $FLAGS -x cu -c "$REF/$f" -o "$OBJ/$f.o" &
        pids+=($!)
      done
      "$NVCC" $FLAGS -x cu -c "$HERE/ref_match_harness.cpp" -o "$OBJ/ref_match_harness.o" &
      pids+=($!)
      for p in "${pids[@]}"; do wait "$p"; done
      LIBOBJS="$OBJ/io.cu.o $OBJ/cpuGraph.cpp.o $OBJ/gpuGraph.cpp.o $OBJ/decycle.cpp.o $OBJ/order.cpp.o $OBJ/structure.cu.o $OBJ/filter.cu.o $OBJ/globals.cu.o $OBJ/join.cu.o"
      "$NVCC" -rdc=true -gencode arch=compute_103a,code=sm_103a $LIBOBJS "$OBJ/main.cu.o" -o "$OUT/ClusterSM" -lcudart -lcuda
      echo "$OUT/ClusterSM"
      "$NVCC" -rdc=true -gencode arch=compute_103a,code=sm_103a $LIBOBJS "$OBJ/ref_match_harness.o" -o "$OUT/ref_match" -lcudart -lcuda
      echo "$OUT/ref_match"
      ;;
    *)
      echo "unknown target $t" >&2
      exit 2
      ;;
  esac
done
