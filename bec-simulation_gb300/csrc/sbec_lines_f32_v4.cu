// FP32 line kernels, variant 4 (plan family 0, tile scale 0, ping-pong stages).
#include "sbec_lines_impl.cuh"

namespace sbec {
template struct LineKernels<float, 4>;
}  // namespace sbec
