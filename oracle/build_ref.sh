#!/usr/bin/env bash
# Compiles, from the reference sources where they lie:
#  - the reference's host-callable pieces (Lattice, Mass, Spring, Vec and the
#    constraint applyForce functions: src/object.cu, src/mass.cu,
#    src/spring.cu, src/vec.cu) plus oracle/ref_host_shim.cu into
#    oracle/_ref/libtitan_ref_host.so;
#  - the reference's device code (the same files and src/sim.cu, whose
#    computeSpringForces / massForcesAndUpdate kernels are the reference's
#    step) plus oracle/ref_gpu_shim.cu, device-linked into
#    oracle/_ref/titan_ref_kernels.cubin for oracle/ref_gpu_harness.cpp.
# Device code keeps nvcc's default contraction (--fmad=true), as the
# reference's own CMake build does (CMakeLists.txt sets no device flags).
# One build flag is added: -maxrregcount=64.  Built as-is for sm_103a,
# massForcesAndUpdate takes 78 registers per thread, so its launch with the
# reference's THREADS_PER_BLOCK = 1024 (include/Titan/sim.h:32) fails with
# "too many resources requested" -- an error the reference's gpuErrchk
# prints and then ignores (src/sim.cu:61-75), stepping nothing.  Capping
# registers keeps the reference's kernels and launch shape unchanged.
# Test infrastructure only; the reference's own build system is not used.
set -euo pipefail
REF=${TITAN_REFERENCE:-/root/reference}
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
NVCC=${NVCC:-nvcc}
[ -f "$REF/src/object.cu" ] || { echo "reference sources not found at $REF (set TITAN_REFERENCE)" >&2; exit 3; }
mkdir -p "$OUT/obj"
FLAGS=(-std=c++17 -O2 -DCONSTRAINTS -rdc=true -maxrregcount=64 -Xcompiler -fPIC,-ffp-contract=off
       -gencode arch=compute_103a,code=sm_103a
       -I "$HERE/ref_shims" -I "$REF/include/Titan" -I "$REF/include"
       -include "$HERE/ref_shims/titan_ref_compat.h" -w)
pids=()
for f in object mass spring vec sim; do
  "$NVCC" "${FLAGS[@]}" -c "$REF/src/$f.cu" -o "$OUT/obj/$f.o" & pids+=($!)
done
"$NVCC" "${FLAGS[@]}" -c "$HERE/ref_host_shim.cu" -o "$OUT/obj/shim.o" & pids+=($!)
"$NVCC" "${FLAGS[@]}" -c "$HERE/ref_gpu_shim.cu" -o "$OUT/obj/gpu_shim.o" & pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
"$NVCC" -shared -rdc=true -gencode arch=compute_103a,code=sm_103a -o "$OUT/libtitan_ref_host.so" \
  "$OUT"/obj/{object,mass,spring,vec,shim}.o -lcudart
# nvlink drops kernels that no host code launches; name the ones the
# harness loads
"$NVCC" -dlink -cubin -gencode arch=compute_103a,code=sm_103a -o "$OUT/titan_ref_kernels.cubin" \
  -Xnvlink=-kernels-used=ref_gpu_ -Xnvlink=-kernels-used=computeSpringForces \
  -Xnvlink=-kernels-used=massForcesAndUpdate \
  "$OUT"/obj/{sim,object,mass,spring,vec,gpu_shim}.o
echo "built $OUT/libtitan_ref_host.so $OUT/titan_ref_kernels.cubin"
