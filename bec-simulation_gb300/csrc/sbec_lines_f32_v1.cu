// FP32 line kernels, variant 1 (plan family 1, tile scale 0).
#include "sbec_lines_impl.cuh"

namespace sbec {
template struct LineKernels<float, 1>;
}  // namespace sbec
