// Kernel registry: every integration kernel is instantiated in its own translation unit
// (k_<precision>_<metric>.cu) and handed to the host library as a function pointer.
#pragma once

#include "engine.h"

namespace foort {

// Returns the __global__ function for (metric, integrator), or nullptr.
const void* fp64_kernel(int metric_id, int integrator);
const void* mixed_kernel(int metric_id, int integrator);
// decide64: terminations and diagnostics decided in FP64 (else in float-float)
const void* mixed_kernel_variant(int metric_id, int integrator, bool decide64);
// two lanes per geodesic, or nullptr where that kernel does not exist
const void* mixed_pair_kernel_variant(int metric_id, int integrator, bool decide64);

// Host-side helpers of the mixed-precision kernels (per-image FP32 constants).
void fill_mixed_constants(int metric_id, ImageConst& ic, const RunConst& rc);

}  // namespace foort
