// FP32 register-resident row passes and strided lines, variant 12 (plan family 0, tile scale 0, ping-pong stages).
#include "sbec_lines_impl.cuh"

namespace sbec {
template struct RegKernels<float, 12>;
}  // namespace sbec
