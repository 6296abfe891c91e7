// FP32 register-resident row passes and strided lines, variant 14 (plan family 0, tile scale 1, ping-pong stages).
#include "sbec_lines_impl.cuh"

namespace sbec {
template struct RegKernels<float, 14>;
}  // namespace sbec
