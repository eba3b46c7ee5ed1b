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
# The grid-key files (octree / quadtree and the two key classes) are built
# through the reference's MSVC branch: the GCC branch of
# matching_leading_bits (src/UIntKey96.h:243-250, src/UIntKey64.h:220-225)
# is an unfinished stub with which the redistribution functions never
# return. ref_compat/intrin.h supplies the one MSVC intrinsic that branch
# calls (_BitScanReverse). No other file of the reference tests __GNUC__ or
# _MSC_VER except accelerators.cpp (a compiler name string), which keeps the
# default flags.
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]
#   REFERENCE_ROOT defaults to $CVTX_REFERENCE_ROOT, else to a directory named
#   "reference" beside this repository.
set -euo pipefail
here="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
repo="$(cd "$here/.." && pwd)"
ref="${1:-${CVTX_REFERENCE_ROOT:-$(cd "$repo/.." && pwd)/reference}}"
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
key_flags=(-U__GNUC__ -D_MSC_VER=1929 -I "$here/ref_compat")
objs=()
pids=()
for src in "$ref"/src/*.cpp; do
  name="$(basename "${src%.cpp}")"
  obj="$out/obj/$name.o"
  objs+=("$obj")
  case "$name" in
    GridParticleOcttree|GridParticleQuadtree|UIntKey96|UIntKey64)
      "$CXX" "${flags[@]}" "${key_flags[@]}" -c "$src" -o "$obj" & ;;
    *)
      "$CXX" "${flags[@]}" -c "$src" -o "$obj" & ;;
  esac
  pids+=($!)
done
for p in "${pids[@]}"; do wait "$p"; done
"$CXX" -shared -fopenmp -o "$out/libcvtx_ref.so" "${objs[@]}"
echo "build_ref: built $out/libcvtx_ref.so"
