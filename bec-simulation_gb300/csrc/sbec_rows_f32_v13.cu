// FP32 register-resident row passes and strided lines, variant 13 (plan family 1, tile scale 0, ping-pong stages).
#include "sbec_lines_impl.cuh"

namespace sbec {
template struct RegKernels<float, 13>;
}  // namespace sbec
