// FP64 instantiation of the persistent 1-D ITP steps.
#include "sbec_itp_steps.cuh"

namespace sbec {
template void row_itp_steps<double>(const LineCtx<double>&, const Tw<double>&, int, int, const RowArgs<double>&,
                                    long long, int, double*);
}  // namespace sbec
