#!/usr/bin/env bash
# Compiles the reference's own host code, where it lies, together with
# oracle/ref/ref_shim.cpp into oracle/_ref/libref.so (TEST INFRASTRUCTURE:
# used to pin the oracle and to generate tests/golden fixtures; never
# committed, never shipped). The reference's .cu element files hold
# __host__ __device__ functions; they are compiled here as plain C++ against
# the CUDA headers (which define those qualifiers away for a host compiler).
# -fpermissive: fem/HexElement.cuh declares EvaluateModal3D* extern while
# fem/HexElement.cu defines them static inline. -include cstdint:
# xml_fld_geometry_builder.cpp uses uint64_t without including it.
# -ffp-contract=off matches the oracle's build so FP32 results can be
# compared bit for bit.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
if [ -z "${HORENDER_REFERENCE:-}" ]; then
  echo "HORENDER_REFERENCE (the reference checkout's root) is not set; skipping" >&2
  exit 0
fi
REF="$HORENDER_REFERENCE/FEM-AABB"
OUT="$HERE/_ref"
if [ ! -d "$REF" ]; then
  echo "reference sources not found at $REF; skipping" >&2
  exit 0
fi
CUDA_INC="${CUDA_HOME:-/usr/local/cuda}/include"
mkdir -p "$OUT/obj"
FLAGS=(-std=c++17 -O2 -fPIC -ffp-contract=off -fpermissive -include cstdint -w -I"$REF" -I"$REF/fem" -I"$CUDA_INC")
SRCS=(BVH.cu fem/HexElement.cu fem/RayIsosurface.cu fem/PrismElement.cu fem/QuadElement.cu fem/TriElement.cu
      xml_fld_loader.cpp xml_fld_common.cpp xml_fld_math.cpp xml_fld_field_parser.cpp
      xml_fld_geometry_parser.cpp xml_fld_geometry_builder.cpp vtu_loader.cpp)
pids=()
objs=()
for s in "${SRCS[@]}"; do
  o="$OUT/obj/$(echo "$s" | tr '/.' '__').o"
  objs+=("$o")
  g++ "${FLAGS[@]}" -x c++ -c "$REF/$s" -o "$o" &
  pids+=($!)
done
g++ "${FLAGS[@]}" -x c++ -c "$HERE/ref/ref_shim.cpp" -o "$OUT/obj/ref_shim.o" &
pids+=($!)
objs+=("$OUT/obj/ref_shim.o")
for p in "${pids[@]}"; do wait "$p"; done
g++ -shared -o "$OUT/libref.so" "${objs[@]}" -lz
echo "built $OUT/libref.so"
