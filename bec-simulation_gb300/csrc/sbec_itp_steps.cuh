// Persistent 1-D ITP steps (k_row_itp_steps) for lines of 32-1024 points, plan variant 0;
// included by one translation unit per precision (sbec_itp_steps_f32.cu / _f64.cu), which
// instantiates row_itp_steps<R>.
#pragma once

#include <string>

#include "sbec_lines_impl.cuh"

namespace sbec {

namespace {

template <typename R, int NN, int D>
void launch_itp_steps(const LineCtx<R>& c, const Tw<R>& tw, const RowArgs<R>& a, long long n_steps,
                      int first_pending, double* norm_out) {
  constexpr int RPB = row_rpb_v<R, NN, D, 0>();
  constexpr int NT = row_threads<R, NN, D, RPB, 0>();
  constexpr long TILE = (long)sizeof(cplx<R>) * D * RPB * NN;
  if constexpr (NT > 1024 || TILE > 200 * 1024) {
    fail(SBEC_ERR_UNSUPPORTED, "row pass tile too large for this line length");
  } else {
    auto kern = k_row_itp_steps<R, NN, D, RPB, 0, false>;
    static const bool once = (line_set_smem(kern, (size_t)TILE), true);
    (void)once;
    line_launch(c, kern, dim3(1), dim3(NT), (size_t)TILE, a, c.st, c.ph, tw, n_steps, first_pending, norm_out);
  }
}

template <typename R, int NN>
void launch_itp_steps_d(const LineCtx<R>& c, const Tw<R>& tw, int D, const RowArgs<R>& a, long long n_steps,
                        int first_pending, double* norm_out) {
  switch (D) {
    case 1: launch_itp_steps<R, NN, 1>(c, tw, a, n_steps, first_pending, norm_out); return;
    case 3: launch_itp_steps<R, NN, 3>(c, tw, a, n_steps, first_pending, norm_out); return;
    case 5: launch_itp_steps<R, NN, 5>(c, tw, a, n_steps, first_pending, norm_out); return;
    default: fail(SBEC_ERR_UNSUPPORTED, "fused path needs D in {1,3,5}");
  }
}

}  // namespace

template <typename R>
void row_itp_steps(const LineCtx<R>& c, const Tw<R>& tw, int n, int D, const RowArgs<R>& a, long long n_steps,
                   int first_pending, double* norm_out) {
  switch (n) {
    case 32: launch_itp_steps_d<R, 32>(c, tw, D, a, n_steps, first_pending, norm_out); return;
    case 64: launch_itp_steps_d<R, 64>(c, tw, D, a, n_steps, first_pending, norm_out); return;
    case 128: launch_itp_steps_d<R, 128>(c, tw, D, a, n_steps, first_pending, norm_out); return;
    case 256: launch_itp_steps_d<R, 256>(c, tw, D, a, n_steps, first_pending, norm_out); return;
    case 512: launch_itp_steps_d<R, 512>(c, tw, D, a, n_steps, first_pending, norm_out); return;
    case 1024: launch_itp_steps_d<R, 1024>(c, tw, D, a, n_steps, first_pending, norm_out); return;
    default: fail(SBEC_ERR_UNSUPPORTED, "no persistent ITP row kernel for length " + std::to_string(n));
  }
}

}  // namespace sbec
