// FFT line kernels (contiguous x lines, strided lines, the fused row pass) in the
// variants the autotuner chooses between.  A variant V combines
//   plan family  V & 1:  0 = the precision's default radix set (FP64 radix-16,
//                            FP32 radix-4/8), 1 = the other one;
//   tile scale   (V >> 1) & 1: 0 = ~64-thread tiles (spread a single small solve
//                            over all SMs), 1 = wider tiles (x lines / row pass
//                            2x the lines per block, strided 4x the columns, i.e.
//                            64-128 contiguous bytes per row segment);
//   stages       V >> 2: 0 = in place (two block barriers per Stockham stage),
//                            1 = ping-pong between two shared tiles (one barrier
//                            per stage, twice the shared memory; x and strided
//                            lines fall back to in place above 200 KB, a row pass
//                            that does not fit is not a candidate).
// FP32 lines of kMinTunedLine points or more have all eight variants, each compiled
// in its own translation unit (sbec_lines_f32_v<V>.cu); FP64 and shorter lines
// have variant 0 only.
//
// The fused row pass and the strided lines have four more variants, 8 + V for ping-pong V
// (12-15): the register-resident forms (k_row_pass_reg, k_fft_strided_reg;
// sbec_rows_f32_v<V>.cu), in which a thread keeps its positions of a line (of all D lines
// of its row, in the row pass) in registers between the transforms.  Row tiles are rows of
// TPL threads (a thread covers all D components of its positions), ~64 threads at tile
// scale 0 and twice that at scale 1; strided tiles are those of variant V - 8.
#pragma once

#include <algorithm>

#include "sbec_engine.h"
#include "sbec_kernels.cuh"

namespace sbec {

constexpr int kLineVariants = 8;
constexpr int kRowVariants = 16;  // row passes and strided lines: 0-7 tile form, 12-15 register form
constexpr int kMinTunedLine = 32;

// A row-pass / strided variant is compiled: the tile forms, and the register forms with
// ping-pong stages.
inline bool row_variant_compiled(int V) { return V < 8 || (V >= 12 && V < kRowVariants); }
inline bool row_variant_reg(int V) { return V >= 8; }

template <typename R>
struct LineCtx {
  cudaStream_t stream;
  bool pdl;
  PhaseRef<R> ph;
  SpinTabs<R> st;
};

template <typename R, int V>
struct LineKernels {
  static void fft_x(const LineCtx<R>& c, const Tw<R>& tw, int n, cplx<R>* data, int64_t n_lines, int mode);
  static void fft_strided(const LineCtx<R>& c, const Tw<R>& tw, int n, cplx<R>* data, int64_t S, int64_t inner,
                          int64_t outer, int64_t outer_stride, int n_in, int n_out, int mode, const int* omap,
                          int oper);
  static void row(const LineCtx<R>& c, const Tw<R>& tw, int n, int D, const RowArgs<R>& a, int blocks);
};

// Register-resident row passes and strided lines (V = 12..15).
template <typename R, int V>
struct RegKernels {
  static void row(const LineCtx<R>& c, const Tw<R>& tw, int n, int D, const RowArgs<R>& a, int blocks);
  static void fft_strided(const LineCtx<R>& c, const Tw<R>& tw, int n, cplx<R>* data, int64_t S, int64_t inner,
                          int64_t outer, int64_t outer_stride, int n_in, int n_out, int mode, const int* omap,
                          int oper);
};

// n fused ITP split steps of a 1-D solve in one launch (k_row_itp_steps, plan variant 0;
// sbec_itp_steps.cu): lines of 32-1024 points, D in {1, 3, 5}.
constexpr int kItpStepsMaxLine = 1024;
template <typename R>
void row_itp_steps(const LineCtx<R>& c, const Tw<R>& tw, int n, int D, const RowArgs<R>& a, long long n_steps,
                   int first_pending, double* norm_out);

// Persistent 2-D leapfrog segments (sbec_segment_f32.cu, kernel k_lf_segment): FP32,
// square grids of 64-512 points per side, D in {1, 3}.  One cooperative launch runs
// n_steps merged leapfrog steps of the default plan.
bool lf_segment_supported(bool fp32, int nx, int ny, int D);
void lf_segment_launch(const LineCtx<float>& c, const Tw<float>& twx, const Tw<float>& twy, const RowArgs<float>& a,
                       int n, int D, long long n_steps, GridBarrier* bar);

// The variant actually compiled for a line of n points.
inline int line_variant(bool fp32, int n, int V) { return (fp32 && n >= kMinTunedLine) ? V : 0; }

// ---- host mirrors of the tile shapes (must match sbec_lines_impl.cuh)
inline int line_tpl(bool fp32, int n, int V) { return std::max(1, n / plan_radix_host(fp32, n, V & 1)); }

inline int row_rpb_host(bool fp32, int n, int D, int V) {
  V = line_variant(fp32, n, V);
  int r = row_variant_reg(V) ? 64 / line_tpl(fp32, n, V) : 64 / (D * line_tpl(fp32, n, V));
  if (r < 1) r = 1;
  return r << ((V >> 1) & 1);
}

inline int row_threads_host(bool fp32, int n, int D, int V) {
  V = line_variant(fp32, n, V);
  const int rpb = row_rpb_host(fp32, n, D, V);
  if (row_variant_reg(V)) return rpb * line_tpl(fp32, n, V);
  const int fft = D * rpb * line_tpl(fp32, n, V);
  const int pts = std::min(rpb * n, 1024);
  return (std::max(fft, pts) + 31) / 32 * 32;
}

inline size_t row_smem_host(bool fp32, int n, int D, int V) {
  const int pp = (line_variant(fp32, n, V) >> 2) & 1;
  const int line = row_variant_reg(line_variant(fp32, n, V)) ? n + n / 16 : n;  // register rows: padded lines
  return (size_t)(fp32 ? 8 : 16) * D * row_rpb_host(fp32, n, D, V) * line << pp;
}

// A row-pass variant can run: at most 1024 threads and 200 KB of shared memory.
inline bool row_variant_ok(bool fp32, int n, int D, int V) {
  return row_threads_host(fp32, n, D, V) <= 1024 && row_smem_host(fp32, n, D, V) <= 200 * 1024;
}

}  // namespace sbec
