// FP64 kernel instantiations for metric kJohannsen.
#include "kernel_fp64.cuh"
#include "kernels.h"

namespace foort {

const void* fp64_kernel_joh(int integrator) {
    if (integrator == FOORT_INTEGRATOR_RK4)
        return reinterpret_cast<const void*>(&integrate_fp64_kernel<kJohannsen, FOORT_INTEGRATOR_RK4>);
    return reinterpret_cast<const void*>(&integrate_fp64_kernel<kJohannsen, FOORT_INTEGRATOR_VERLET>);
}

}  // namespace foort
