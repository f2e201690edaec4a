// step_var.cu -- register-capped launch-bound variants of the per-tile step
// kernel for the FP32 forms with the Euler integrator (a separate
// translation unit so that the build compiles them in parallel with step.cu).
//   variant 1: __launch_bounds__(256, 3)  <= 85 registers per thread
//   variant 2: __launch_bounds__(256, 4)  <= 64 registers per thread
#include "step_kernel.cuh"

namespace tg {

const void *step_kernel_capped(int precision, int variant) {
    if (precision == P_FP32) {
        if (variant == 1) return (const void *)k_step<P_FP32, 256, 3, INTEG_EULER>;
        if (variant == 2) return (const void *)k_step<P_FP32, 256, 4, INTEG_EULER>;
    } else if (precision == P_FP32C) {
        if (variant == 1) return (const void *)k_step<P_FP32C, 256, 3, INTEG_EULER>;
        if (variant == 2) return (const void *)k_step<P_FP32C, 256, 4, INTEG_EULER>;
    }
    return nullptr;
}

}  // namespace tg
