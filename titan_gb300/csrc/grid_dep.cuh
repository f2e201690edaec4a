// grid_dep.cuh -- programmatic dependent launch between consecutive step
// kernels (launched with cudaLaunchAttributeProgrammaticStreamSerialization,
// captured into the step graphs).  launch_dependents lets the next grid start
// launching; wait blocks until the preceding grid has completed and its
// writes are visible (a no-op when the launch has no programmatic
// predecessor).  A kernel reads only data no step writes before its wait.
// Used by the persistent warp-specialised kernel (one CTA per SM, all
// resident from the start); the per-tile kernel, whose grids hold more CTAs
// than fit at once, measured slower with it (20^3 lattice, FP64: 60 us per
// step against 38), as early-launched dependents take SM slots.
#pragma once

#include <cuda_runtime.h>

namespace tg {
namespace {

__device__ __forceinline__ void grid_dep_launch_dependents() {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
__device__ __forceinline__ void grid_dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// cudaLaunchKernelExC with programmatic stream serialisation allowed
inline cudaError_t launch_programmatic(const void *f, dim3 grid, dim3 block, void **args, size_t smem,
                                       cudaStream_t s) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelExC(&cfg, f, args);
}

}  // namespace
}  // namespace tg
