#!/usr/bin/env bash
# Build the reference's own CPU LBVH / BVH code as a test oracle and CPU
# baseline: oracle/_ref/libref.so.
#
# The sources are compiled where they lie under the reference checkout
# (default /root/reference, override with RT_REFERENCE_DIR); nothing is
# copied into this repository.  Two adaptations are needed to build the
# Windows/MSVC sources with g++:
#   * LBVH.cpp:1577-1578 define bsf/bsr with MSVC inline assembly.  The
#     file is fed to g++ through a stream edit that turns exactly those two
#     definitions into declarations; oracle/ref/ref_shim.cpp defines them
#     with __builtin_ctz/__builtin_clz.
#   * Material.h pulls in Direct3D headers; oracle/ref/shim/ provides empty
#     stand-ins for D3DResource.h and Texture2D.h.
# The vendored OBJ loader (Common/Scenes/Loaders/model_obj.cpp) builds as is.
# Model::Scale is taken out of Common/Scenes/Model.cpp (the function's own
# lines, found by its signature) and compiled against
# oracle/ref/shim/model_scale_stub.h, a Model declaration holding only the
# vertex array, since Model.h itself needs Direct3D.
# Floating point: -O2 -ffp-contract=off (no fused multiply-add), as the
# reference's x86 SSE build would evaluate it.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
ORACLE="$(dirname "$HERE")"
REF="${RT_REFERENCE_DIR:-/root/reference}"
OUT="$ORACLE/_ref"
if [ ! -f "$REF/AccelerationStructures/LBVH/LBVH.cpp" ]; then
  echo "build_ref.sh: reference sources not found under $REF; skipping" >&2
  exit 0
fi
mkdir -p "$OUT"
CXX="${CXX:-g++}"
FLAGS=(-O2 -ffp-contract=off -fPIC -fpermissive -w -fopenmp "-D__int64=long long" -DLINUX
       -include cstdio -include cstring
       -I"$HERE/shim" -I"$REF/Common" -I"$REF/Common/Geometry" -I"$REF/Common/Scenes"
       -I"$REF/AccelerationStructures" -I"$REF/AccelerationStructures/LBVH"
       -I"$REF/AccelerationStructures/BVH" -I"$REF/Common/Scenes/Loaders")
sed -e '1577,1578s/{ *__asm.*}/;/' "$REF/AccelerationStructures/LBVH/LBVH.cpp" \
  | "$CXX" -x c++ "${FLAGS[@]}" -c -o "$OUT/LBVH.o" - &
"$CXX" "${FLAGS[@]}" -c "$REF/AccelerationStructures/BVH/bvh.cpp" -o "$OUT/bvh.o" &
"$CXX" "${FLAGS[@]}" -c "$REF/AccelerationStructures/AccelerationStructure.cpp" -o "$OUT/AccelerationStructure.o" &
"$CXX" "${FLAGS[@]}" -c "$REF/Common/Scenes/Primitive.cpp" -o "$OUT/Primitive.o" &
"$CXX" "${FLAGS[@]}" -c "$REF/Common/Memory.cpp" -o "$OUT/Memory.o" &
"$CXX" "${FLAGS[@]}" -c "$REF/Common/Scenes/Loaders/model_obj.cpp" -o "$OUT/model_obj.o" &
sed -n '/^void Model::Scale()/,/^}/p' "$REF/Common/Scenes/Model.cpp" \
  | "$CXX" -x c++ "${FLAGS[@]}" -include model_scale_stub.h -c -o "$OUT/model_scale.o" - &
"$CXX" "${FLAGS[@]}" -c "$HERE/ref_shim.cpp" -o "$OUT/ref_shim.o" &
wait
"$CXX" -shared -fopenmp -o "$OUT/libref.so" "$OUT/LBVH.o" "$OUT/bvh.o" "$OUT/AccelerationStructure.o" \
  "$OUT/Primitive.o" "$OUT/Memory.o" "$OUT/model_obj.o" "$OUT/model_scale.o" "$OUT/ref_shim.o"
echo "built $OUT/libref.so"
