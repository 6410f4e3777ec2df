// Mixed-precision kernels (placeholder until the FP32 plugins land).
#include "kernels.h"

namespace foort {

const void* mixed_kernel(int, int) { return nullptr; }
void fill_mixed_constants(int, ImageConst&, const RunConst&) {}

}  // namespace foort
