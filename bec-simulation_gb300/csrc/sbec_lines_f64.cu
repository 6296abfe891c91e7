// FP64 line kernels (variant 0 only).
#include "sbec_lines_impl.cuh"

namespace sbec {
template struct LineKernels<double, 0>;
}  // namespace sbec
