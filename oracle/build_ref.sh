#!/usr/bin/env bash
# Compile the UNMODIFIED gpudem CPU step path, where its sources lie, together
# with oracle/ref_harness.cu into oracle/_ref/librefharness.so.  Test
# infrastructure only: used to make and check the golden vectors under
# tests/golden/.  Needs the reference checkout (default /root/reference);
# exits 0 without building when it is absent (e.g. on the GPU host).
#
# Flags follow the reference makefile (makefile:3-5) with the two changes the
# oracle needs: host code without FMA contraction (-ffp-contract=off) and a
# CUDA-13-accepted virtual arch for the device code it carries but never runs.
#
# `build_ref.sh --where` prints the reference checkout this recipe uses
# (GDEM_REFERENCE_DIR, else the default below) and nothing when it is absent;
# the scripts and tests that read reference files ask it.
set -euo pipefail
REF="${GDEM_REFERENCE_DIR:-/root/reference}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ "${1:-}" = "--where" ]; then
  if [ -f "$REF/cpu_dem.cu" ]; then echo "$REF"; fi
  exit 0
fi
if [ ! -f "$REF/cpu_dem.cu" ]; then
  echo "build_ref: no reference sources at $REF; skipping"
  exit 0
fi
mkdir -p "$OUT/obj"
NVCC="${NVCC:-nvcc}"
FLAGS=(-O3 -DUSE_GPU=1 -fmad=false -std=c++17
       -gencode arch=compute_100,code=compute_100
       -Xcompiler "-fopenmp -ffp-contract=off -fPIC -w"
       -I"$REF")
SRCS=(cpu_dem.cu BoundingBox.cu BVH.cu TriangleMesh.cu ParticleSystem.cu)
pids=()
for s in "${SRCS[@]}"; do
  o="$OUT/obj/${s%.cu}.o"
  if [ ! -f "$o" ] || [ "$REF/$s" -nt "$o" ]; then
    "$NVCC" "${FLAGS[@]}" -x cu -c "$REF/$s" -o "$o" &
    pids+=($!)
  fi
done
if [ ! -f "$OUT/obj/cJSON_d.o" ]; then
  gcc -O3 -fPIC -ffp-contract=off -c "$REF/cJSON_d.c" -o "$OUT/obj/cJSON_d.o" &
  pids+=($!)
fi
"$NVCC" "${FLAGS[@]}" -x cu -c "$HERE/ref_harness.cu" -o "$OUT/obj/ref_harness.o" &
pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
"$NVCC" -shared -gencode arch=compute_100,code=compute_100 -Xcompiler "-fopenmp -fPIC" \
  "$OUT"/obj/*.o -o "$OUT/librefharness.so" -lgomp
echo "build_ref: built $OUT/librefharness.so"
