// FP32 line kernels, variant 5 (plan family 1, tile scale 0, ping-pong stages).
#include "sbec_lines_impl.cuh"

namespace sbec {
template struct LineKernels<float, 5>;
}  // namespace sbec
