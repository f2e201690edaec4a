// step.cu -- host side of the per-tile step kernel (step_kernel.cuh): the
// FP64 form and the default launch bounds of every precision; the
// register-capped variants of the FP32 forms are in step_var.cu.
#include <cstdint>
#include <map>
#include <mutex>
#include <utility>

#include "step_kernel.cuh"

namespace tg {

cudaError_t raise_smem_limit(const void *f, size_t smem) {
    static std::mutex mu;
    static std::map<std::pair<int, const void *>, size_t> limit;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    size_t &cur = limit[{dev, f}];
    if (smem <= cur) return cudaSuccess;
    e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) cur = smem;
    return e;
}

int state_words(int precision) { return precision == P_FP64 ? 6 : (precision == P_FP32C ? 12 : 8); }
int state_record_bytes(int precision) { return precision == P_FP32 ? 32 : 48; }
int entry_record_bytes(int precision) { return precision == P_FP64 ? 32 : 16; }

size_t tile_smem_bytes(int precision, int slots, int entries, int heavy) {
    const int64_t rec = precision == P_FP32 ? 32 : 48;
    const int64_t slot = precision == P_FP64 ? 32 : 16;
    const int64_t rs = precision == P_FP64 ? 8 : 4;
    return (size_t)(align16((int64_t)slots * rec) + (int64_t)entries * slot + 3 * (int64_t)heavy * rs);
}

template <int PREC>
const void *step_kernel_default(int integ) {
    switch (integ) {
        case INTEG_VERLET: return (const void *)k_step<PREC, 512, 1, INTEG_VERLET>;
        case INTEG_RK2: return (const void *)k_step<PREC, 512, 1, INTEG_RK2>;
        default: return (const void *)k_step<PREC, 512, 1, INTEG_EULER>;
    }
}

// The register-capped variants exist for Euler in the FP32 forms; other
// requests run the default launch bounds.
const void *step_kernel(int precision, int variant, int integ) {
    if (variant != 0 && precision != P_FP64 && integ == INTEG_EULER) return step_kernel_capped(precision, variant);
    return precision == P_FP64   ? step_kernel_default<P_FP64>(integ)
           : precision == P_FP32 ? step_kernel_default<P_FP32>(integ)
                                 : step_kernel_default<P_FP32C>(integ);
}

cudaError_t step_prepare(int precision, int variant, int integ, size_t smem) {
    const void *f = step_kernel(precision, variant, integ);
    if (!f) return cudaErrorInvalidValue;
    return raise_smem_limit(f, smem);
}

cudaError_t launch_step(int precision, int variant, int integ, const StepArgs &a, int ntiles, int threads,
                        size_t smem, int parity, int write_acc, cudaStream_t s) {
    if (ntiles <= 0) return cudaSuccess;
    const void *f = step_kernel(precision, variant, integ);
    if (!f) return cudaErrorInvalidValue;
    void *args[] = {const_cast<StepArgs *>(&a), &parity, &write_acc};
    return cudaLaunchKernel(f, dim3(ntiles), dim3(threads), args, smem, s);
}

}  // namespace tg
