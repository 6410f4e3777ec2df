// FP64 kernel instantiations for metric kRasheedLarsen.
#include "kernel_fp64.cuh"
#include "kernels.h"

namespace foort {

const void* fp64_kernel_rl(int integrator) {
    if (integrator == FOORT_INTEGRATOR_RK4)
        return reinterpret_cast<const void*>(&integrate_fp64_kernel<kRasheedLarsen, FOORT_INTEGRATOR_RK4>);
    return reinterpret_cast<const void*>(&integrate_fp64_kernel<kRasheedLarsen, FOORT_INTEGRATOR_VERLET>);
}

}  // namespace foort
