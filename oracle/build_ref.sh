#!/usr/bin/env bash
# Compiles the reference's host-callable pieces (Lattice, Mass, Spring, Vec and
# the constraint applyForce functions: src/object.cu, src/mass.cu,
# src/spring.cu, src/vec.cu) from the reference sources where they lie, plus
# oracle/ref_host_shim.cu, into oracle/_ref/libtitan_ref_host.so.
# Test infrastructure only; the reference's own build system is not used.
set -euo pipefail
REF=${TITAN_REFERENCE:-/root/reference}
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
NVCC=${NVCC:-nvcc}
[ -f "$REF/src/object.cu" ] || { echo "reference sources not found at $REF" >&2; exit 1; }
mkdir -p "$OUT/obj"
FLAGS=(-std=c++17 -O2 -DCONSTRAINTS -rdc=true -Xcompiler -fPIC,-ffp-contract=off
       -gencode arch=compute_103a,code=sm_103a
       -I "$HERE/ref_shims" -I "$REF/include/Titan" -I "$REF/include"
       -include "$HERE/ref_shims/titan_ref_compat.h" -w)
pids=()
for f in object mass spring vec; do
  "$NVCC" "${FLAGS[@]}" -c "$REF/src/$f.cu" -o "$OUT/obj/$f.o" & pids+=($!)
done
"$NVCC" "${FLAGS[@]}" -c "$HERE/ref_host_shim.cu" -o "$OUT/obj/shim.o" & pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
"$NVCC" -shared -rdc=true -gencode arch=compute_103a,code=sm_103a -o "$OUT/libtitan_ref_host.so" \
  "$OUT"/obj/{object,mass,spring,vec,shim}.o -lcudart
echo "built $OUT/libtitan_ref_host.so"
