// Mixed-precision kernel instantiations for metric kRasheedLarsen.
#include "kernel_mixed.cuh"
#include "kernels.h"

namespace foort {

template <int MID, int INTEG, bool D64>
// At most 168 registers, so that three CTAs fit on an SM: on GB300 samples of 100,000
// geodesics of the Johannsen Verlet 1024² run and of the Kerr a = 0.998 adaptive run run
// 1.20x and 1.29x faster than with
// the 255 / 128 registers of two CTAs, and faster than four CTAs' 128 with their spills.
__global__ void __launch_bounds__(128, 3) integrate_mixed_kernel(const __grid_constant__ LaunchArgs A,
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
