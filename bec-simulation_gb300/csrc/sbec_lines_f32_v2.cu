// FP32 line kernels, variant 2 (plan family 0, tile scale 1).
#include "sbec_lines_impl.cuh"

namespace sbec {
template struct LineKernels<float, 2>;
}  // namespace sbec
