// FP32 line kernels, variant 6 (plan family 0, tile scale 1, ping-pong stages).
#include "sbec_lines_impl.cuh"

namespace sbec {
template struct LineKernels<float, 6>;
}  // namespace sbec
