#!/bin/bash
# Builds the reference (ADEPT / GPU-BSW) driver and kernels for sm_103a from the
# reference's own source files, linked with oracle/ref_harness.cpp, into
# oracle/_ref/ref_harness.  Test infrastructure: the binary is the reference
# side of the differential checks and of the GPU-vs-reference timing.
#
# The reference's CMake recipe does not build under CUDA 13 (its gencode list
# starts at compute_50), so the four translation units are compiled directly
# with nvcc.  driver.cpp needs -std=c++17 because CUDA 13's thrust headers
# (included but unused at driver.cpp:6-8) reject C++14.
#
# Where the reference tree is present (GBSW_REFERENCE_DIR, by default a
# checkout named "reference" beside this repository) its eight
# driver/kernel/utils/alignments sources are staged
# into oracle/_ref/src first; oracle/_ref/ is git-ignored, so the staged copy
# only travels with the working tree to a GPU host, where the build runs
# again from it.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/_ref"
SRC="${GBSW_REFERENCE_DIR:-$(cd "$HERE/../.." && pwd)/reference}"
NVCC="${NVCC:-nvcc}"
mkdir -p "$OUT/src" "$OUT/obj"
if [ -d "$SRC" ]; then
  for f in alignments.cpp alignments.hpp driver.cpp driver.hpp kernel.cpp kernel.hpp utils.cpp utils.hpp; do
    cp -f "$SRC/$f" "$OUT/src/$f"
    chmod u+w "$OUT/src/$f"
  done
fi
if [ ! -f "$OUT/src/kernel.cpp" ]; then
  echo "build_ref.sh: no reference sources (set GBSW_REFERENCE_DIR)" >&2
  exit 3
fi
ARCH="-gencode arch=compute_103a,code=sm_103a"
FLAGS="$ARCH -O3 -Xcompiler -fopenmp -I$OUT/src"
pids=()
"$NVCC" $FLAGS -std=c++14 -x cu -c "$OUT/src/kernel.cpp" -o "$OUT/obj/kernel.o" & pids+=($!)
"$NVCC" $FLAGS -std=c++17 -x cu -c "$OUT/src/driver.cpp" -o "$OUT/obj/driver.o" & pids+=($!)
"$NVCC" $FLAGS -std=c++14 -x cu -c "$OUT/src/utils.cpp" -o "$OUT/obj/utils.o" & pids+=($!)
"$NVCC" $FLAGS -std=c++14 -x cu -c "$OUT/src/alignments.cpp" -o "$OUT/obj/alignments.o" & pids+=($!)
"$NVCC" $FLAGS -std=c++17 -DGBSW_REF_WRAP_LAUNCH -x cu -c "$HERE/ref_harness.cpp" -o "$OUT/obj/ref_harness.o" & pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
# every kernel launch of the reference's objects goes through the harness's
# event-bracketing wrapper (its kernel time; see ref_harness.cpp)
"$NVCC" $ARCH -Xcompiler -fopenmp -Xlinker --wrap=__cudaLaunchKernel -o "$OUT/ref_harness" "$OUT"/obj/*.o -lgomp
echo "$OUT/ref_harness"
