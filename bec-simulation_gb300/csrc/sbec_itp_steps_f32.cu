// FP32 instantiation of the persistent 1-D ITP steps.
#include "sbec_itp_steps.cuh"

namespace sbec {
template void row_itp_steps<float>(const LineCtx<float>&, const Tw<float>&, int, int, const RowArgs<float>&, long long,
                                   int, double*);
}  // namespace sbec
