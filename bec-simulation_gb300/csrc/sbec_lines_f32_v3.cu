// FP32 line kernels, variant 3 (plan family 1, tile scale 1).
#include "sbec_lines_impl.cuh"

namespace sbec {
template struct LineKernels<float, 3>;
}  // namespace sbec
