// Mixed-precision kernel instantiations for metric kRasheedLarsen.
#include "kernel_mixed.cuh"
#include "kernels.h"

namespace foort {

template <int MID, int INTEG, bool D64>
__global__ void __launch_bounds__(128) integrate_mixed_kernel(const __grid_constant__ LaunchArgs A,
                                                              const __grid_constant__ RunConst R) {
    persistent_loop<MixedEngine<MID, INTEG, D64>>(A, R);
}

const void* mixed_kernel_rl(int integrator, bool decide64) {
    if (integrator == FOORT_INTEGRATOR_RK4)
        return decide64 ? reinterpret_cast<const void*>(&integrate_mixed_kernel<kRasheedLarsen, FOORT_INTEGRATOR_RK4, true>)
                        : reinterpret_cast<const void*>(&integrate_mixed_kernel<kRasheedLarsen, FOORT_INTEGRATOR_RK4, false>);
    return decide64 ? reinterpret_cast<const void*>(&integrate_mixed_kernel<kRasheedLarsen, FOORT_INTEGRATOR_VERLET, true>)
                    : reinterpret_cast<const void*>(&integrate_mixed_kernel<kRasheedLarsen, FOORT_INTEGRATOR_VERLET, false>);
}

}  // namespace foort
