// FP32 line kernels, variant 7 (plan family 1, tile scale 1, ping-pong stages).
#include "sbec_lines_impl.cuh"

namespace sbec {
template struct LineKernels<float, 7>;
}  // namespace sbec
