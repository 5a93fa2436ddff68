#!/bin/bash
# ORACLE -- test infrastructure only.
# Builds oracle/_ref/libref_cpu.so from the reference's own CPU test sources where
# they lie (the reference tree's root: the first argument, else REF_ROOT; one of them
# is required), compiled against the stand-in
# headers in oracle/ref_shim/ (Armadillo pinv and Boost normal cdf restated), plus
# oracle/ref_harness.cpp. Used only to pin the oracle and to make the golden
# fixtures; the reference tree is not present where the GPU tests run. The
# reference relies on Armadillo to pull in <memory> and friends, so those standard
# headers are force-included (-include) instead of editing its sources.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF_ROOT="${1:-${REF_ROOT:-}}"
[ -n "$REF_ROOT" ] || { echo "usage: build_ref.sh <reference tree root> (or set REF_ROOT)" >&2; exit 2; }
SRC="$REF_ROOT/src"
OUT="$HERE/_ref"
[ -d "$SRC" ] || { echo "reference sources not found at $SRC" >&2; exit 2; }
mkdir -p "$OUT"
CXXFLAGS="-include memory -include string -include sstream -include fstream -include cstring -O2 -std=c++17 -fPIC -fopenmp -ffp-contract=off -DWITH_CUDA_ATOMICS=0 -DMIGRATE_EDGES=0 -DNDEBUG"
INC="-I$HERE/ref_shim -I$SRC -I/usr/local/cuda/include"
pids=()
for f in executor/cpuExecutor.cpp executor/testing/cpuRowTests.cpp executor/testing/cpuUtil.cpp \
         executor/testing/cpuWorkstealingTests.cpp executor/independence/cpuInd.cpp; do
  o="$OUT/$(basename "$f" .cpp).o"
  g++ $CXXFLAGS $INC -w -c "$SRC/$f" -o "$o" & pids+=($!)
done
# binomialCoeff / ithCombination (host+device functions) from the CUDA utility file
nvcc -std=c++17 -O2 -Xcompiler -fPIC -Xcompiler -ffp-contract=off -gencode arch=compute_103a,code=sm_103a \
     -w -c "$SRC/util/cuda_util.cu" -o "$OUT/cuda_util.o" & pids+=($!)
g++ $CXXFLAGS $INC -c "$HERE/ref_harness.cpp" -o "$OUT/ref_harness.o" & pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
g++ -shared -fopenmp -o "$OUT/libref_cpu.so" "$OUT"/*.o -L/usr/local/cuda/lib64 -lcudart
echo "built $OUT/libref_cpu.so"
