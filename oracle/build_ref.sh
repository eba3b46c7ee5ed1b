#!/usr/bin/env bash
# Builds the reference cvortex CPU path (OpenMP, OpenCL off) from the reference
# sources where they lie, into oracle/_ref/libcvtx_ref.so. Test infrastructure
# only: the product never links or loads this library.
#
# The reference depends on the external small-vector library "bsv" (not shipped
# with it, no version pin: reference CMakeLists.txt:69-71); the stand-in header
# under include/bsv/ supplies the types and helpers it uses. Two flags are
# needed beyond the reference's own CMake options (CMakeLists.txt:8-54):
#   -fpermissive  for the extra qualification at src/UIntKey96.h:122 and
#                 src/UIntKey64.h:114, which g++ 13 rejects otherwise;
#   -DNDEBUG      so that viscous calls with singular/planetary regularisation
#                 print a warning and return zeros (src/VortFunc.cpp:52-62)
#                 instead of aborting on assert(0).
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]   (default /root/reference)
set -euo pipefail
here="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
repo="$(cd "$here/.." && pwd)"
ref="${1:-/root/reference}"
out="$here/_ref"
if [ ! -d "$ref/src" ]; then
  echo "build_ref: reference sources not found at $ref; skipping" >&2
  exit 0
fi
mkdir -p "$out/obj"
CXX="${CXX:-g++}"
flags=(-std=c++17 -O3 -DNDEBUG -fPIC -fopenmp -fpermissive -w
       -DCVTX_USING_OPENMP "-DCVTX_EXPORT=" -DCVORTEX_VERSION_MAJOR=0
       -DCVORTEX_VERSION_MINOR=3 -DCVORTEX_VERSION_PATCH=8
       -I "$repo/include" -I "$ref/include/cvortex")
objs=()
pids=()
for src in "$ref"/src/*.cpp; do
  obj="$out/obj/$(basename "${src%.cpp}").o"
  objs+=("$obj")
  "$CXX" "${flags[@]}" -c "$src" -o "$obj" &
  pids+=($!)
done
for p in "${pids[@]}"; do wait "$p"; done
"$CXX" -shared -fopenmp -o "$out/libcvtx_ref.so" "${objs[@]}"
echo "build_ref: built $out/libcvtx_ref.so"
