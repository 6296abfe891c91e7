// FP32 line kernels, variant 0 (plan family 0, tile scale 0).
#include "sbec_lines_impl.cuh"

namespace sbec {
template struct LineKernels<float, 0>;
}  // namespace sbec
