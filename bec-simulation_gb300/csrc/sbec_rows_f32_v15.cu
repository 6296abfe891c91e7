// FP32 register-resident row passes and strided lines, variant 15 (plan family 1, tile scale 1, ping-pong stages).
#include "sbec_lines_impl.cuh"

namespace sbec {
template struct RegKernels<float, 15>;
}  // namespace sbec
