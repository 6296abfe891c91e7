// Definitions of LineKernels<R, V>: tile shapes of each variant and the launch
// switch over line lengths.  Included by one translation unit per (precision,
// variant), which instantiates LineKernels<R, V> explicitly.
#pragma once

#include <string>

#include "sbec_lines.h"

namespace sbec {

template <typename K>
inline void line_set_smem(K kernel, size_t bytes) {
  // opt in above 40 KB: dynamic plus the kernels' static shared arrays must fit the limit
  if (bytes > 40 * 1024)
    cuda_check(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes),
               "cudaFuncSetAttribute");
}

template <typename R, typename... KArgs, typename... Args>
inline void line_launch(const LineCtx<R>& c, void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem,
                        Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = c.stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = c.pdl ? 1 : 0;
  cuda_check(cudaLaunchKernelEx(&cfg, kern, args...), "cudaLaunchKernelEx");
}

// ---- tile shapes (host mirrors in sbec_lines.h)
template <typename R, int N, int V>
constexpr int x_lpb_v() {
  constexpr int tpl = N / PlanOf<R, N, (V & 1)>::E;
  constexpr int lpb = 64 / tpl;
  return (lpb < 1 ? 1 : lpb) << ((V >> 1) & 1);
}

// Ping-pong stages for variants with bit 2 set, where the two tiles fit in 200 KB.
constexpr bool line_pp_v(int V, long tile_bytes) { return ((V >> 2) & 1) && 2 * tile_bytes <= 200 * 1024; }

// Strided tiles: at least 16 contiguous bytes per row segment, ~64 threads at
// scale 0, 4x the columns at scale 1; capped at 1024 threads and 96 KB.
template <typename R, int N, int V>
constexpr int strided_w_v() {
  constexpr int tpl = N / PlanOf<R, N, (V & 1)>::E;
  constexpr int seg = 16 / (int)sizeof(cplx<R>);
  int w = 64 / tpl;
  if (w < seg) w = seg;
  w <<= 2 * ((V >> 1) & 1);
  while (w > 1 && (w * tpl > 1024 || (long)w * N * (int)sizeof(cplx<R>) > 96 * 1024)) w /= 2;
  return w;
}

template <typename R, int N, int D, int V>
constexpr int row_rpb_v() {
  constexpr int tpl = N / PlanOf<R, N, (V & 1)>::E;
  constexpr int r = 64 / (D * tpl);
  return (r < 1 ? 1 : r) << ((V >> 1) & 1);
}

template <typename R, int V>
struct LineImpl {
  static constexpr int P = V & 1;

  template <int NN>
  static void fft_x(const LineCtx<R>& c, const Tw<R>& tw, cplx<R>* data, int64_t n_lines, int mode) {
    constexpr int LPB = x_lpb_v<R, NN, V>();
    constexpr int TPL = NN / PlanOf<R, NN, P>::E;
    constexpr long TILE = (long)sizeof(cplx<R>) * LPB * NN;
    constexpr bool PP = line_pp_v(V, TILE);
    const size_t smem = PP ? 2 * TILE : TILE;
    auto kern = k_fft_x<R, NN, LPB, P, PP>;
    static const bool once = (line_set_smem(kern, smem), true);
    (void)once;
    const int64_t blocks = (n_lines + LPB - 1) / LPB;
    line_launch(c, kern, dim3((unsigned)blocks), dim3(LPB * TPL), smem, data, n_lines, mode, c.ph, tw);
  }

  template <int NN>
  static void fft_strided(const LineCtx<R>& c, const Tw<R>& tw, cplx<R>* data, int64_t S, int64_t inner,
                          int64_t outer, int64_t outer_stride, int n_in, int n_out, int mode, const int* omap,
                          int oper) {
    constexpr int W = strided_w_v<R, NN, V>();
    constexpr int TPL = NN / PlanOf<R, NN, P>::E;
    constexpr long TILE = (long)sizeof(cplx<R>) * W * NN;
    constexpr bool PP = line_pp_v(V, TILE);
    const size_t smem = PP ? 2 * TILE : TILE;
    auto kern = k_fft_strided<R, NN, W, P, PP>;
    static const bool once = (line_set_smem(kern, smem), true);
    (void)once;
    dim3 grid((unsigned)((inner + W - 1) / W), (unsigned)outer);
    line_launch(c, kern, grid, dim3(W * TPL), smem, data, S, inner, outer_stride, n_in, n_out, mode, c.ph, tw, omap,
                oper);
  }

  template <int NN, int D>
  static void row(const LineCtx<R>& c, const Tw<R>& tw, const RowArgs<R>& a, int blocks) {
    constexpr int RPB = row_rpb_v<R, NN, D, V>();
    constexpr int NT = row_threads<R, NN, D, RPB, P>();
    constexpr long TILE = (long)sizeof(cplx<R>) * D * RPB * NN;
    constexpr bool PP = ((V >> 2) & 1) != 0;
    if constexpr (NT > 1024 || (PP ? 2 * TILE : TILE) > 200 * 1024) {
      fail(SBEC_ERR_UNSUPPORTED, "row pass tile too large for this line length");
    } else {
      const size_t smem = PP ? 2 * TILE : TILE;
      auto kern = k_row_pass<R, NN, D, RPB, P, PP>;
      static const bool once = (line_set_smem(kern, smem), true);
      (void)once;
      line_launch(c, kern, dim3((unsigned)blocks), dim3(NT), smem, a, c.st, c.ph, tw);
    }
  }

  template <int NN>
  static void row_n(const LineCtx<R>& c, const Tw<R>& tw, int D, const RowArgs<R>& a, int blocks) {
    switch (D) {
      case 1: row<NN, 1>(c, tw, a, blocks); break;
      case 3: row<NN, 3>(c, tw, a, blocks); break;
      case 5: row<NN, 5>(c, tw, a, blocks); break;
      default: fail(SBEC_ERR_UNSUPPORTED, "fused path needs D in {1,3,5}");
    }
  }
};

#define SBEC_LINE_CASES(FN, ...)                                                           \
  switch (n) {                                                                             \
    case 32: LineImpl<R, V>::template FN<32>(__VA_ARGS__); return;                         \
    case 64: LineImpl<R, V>::template FN<64>(__VA_ARGS__); return;                         \
    case 128: LineImpl<R, V>::template FN<128>(__VA_ARGS__); return;                       \
    case 256: LineImpl<R, V>::template FN<256>(__VA_ARGS__); return;                       \
    case 512: LineImpl<R, V>::template FN<512>(__VA_ARGS__); return;                       \
    case 1024: LineImpl<R, V>::template FN<1024>(__VA_ARGS__); return;                     \
    default: break;                                                                        \
  }                                                                                        \
  if constexpr (V == 0) {                                                                  \
    switch (n) {                                                                           \
      case 2: LineImpl<R, V>::template FN<2>(__VA_ARGS__); return;                         \
      case 4: LineImpl<R, V>::template FN<4>(__VA_ARGS__); return;                         \
      case 8: LineImpl<R, V>::template FN<8>(__VA_ARGS__); return;                         \
      case 16: LineImpl<R, V>::template FN<16>(__VA_ARGS__); return;                       \
      default: break;                                                                      \
    }                                                                                      \
  }

template <typename R, int V>
void LineKernels<R, V>::fft_x(const LineCtx<R>& c, const Tw<R>& tw, int n, cplx<R>* data, int64_t n_lines,
                              int mode) {
  SBEC_LINE_CASES(fft_x, c, tw, data, n_lines, mode)
  switch (n) {
    case 2048: LineImpl<R, V>::template fft_x<2048>(c, tw, data, n_lines, mode); return;
    case 4096: LineImpl<R, V>::template fft_x<4096>(c, tw, data, n_lines, mode); return;
    default: fail(SBEC_ERR_UNSUPPORTED, "unsupported FFT length " + std::to_string(n) + " for line variant " +
                                            std::to_string(V));
  }
}

template <typename R, int V>
void LineKernels<R, V>::fft_strided(const LineCtx<R>& c, const Tw<R>& tw, int n, cplx<R>* data, int64_t S,
                                    int64_t inner, int64_t outer, int64_t outer_stride, int n_in, int n_out,
                                    int mode, const int* omap, int oper) {
  SBEC_LINE_CASES(fft_strided, c, tw, data, S, inner, outer, outer_stride, n_in, n_out, mode, omap, oper)
  fail(SBEC_ERR_UNSUPPORTED, "unsupported strided FFT length " + std::to_string(n) + " for line variant " +
                                 std::to_string(V));
}

template <typename R, int V>
void LineKernels<R, V>::row(const LineCtx<R>& c, const Tw<R>& tw, int n, int D, const RowArgs<R>& a, int blocks) {
  SBEC_LINE_CASES(row_n, c, tw, D, a, blocks)
  switch (n) {
    case 2048: LineImpl<R, V>::template row_n<2048>(c, tw, D, a, blocks); return;
    case 4096: LineImpl<R, V>::template row_n<4096>(c, tw, D, a, blocks); return;
    default: fail(SBEC_ERR_UNSUPPORTED, "unsupported row length " + std::to_string(n) + " for line variant " +
                                            std::to_string(V));
  }
}

#undef SBEC_LINE_CASES

// ---- register-resident row passes and strided lines (V = 12..15: plan V & 1, tile scale
// (V >> 1) & 1, ping-pong)
template <typename R, int N, int V>
constexpr int row_rpb_reg_v() {
  constexpr int tpl = N / PlanOf<R, N, (V & 1)>::E;
  constexpr int r = 64 / tpl;
  return (r < 1 ? 1 : r) << ((V >> 1) & 1);
}

template <typename R, int V>
struct RegImpl {
  static constexpr int P = V & 1;
  static_assert(V >= 12 && V < 16, "register forms are variants 12-15");

  template <int NN>
  static void fft_strided(const LineCtx<R>& c, const Tw<R>& tw, cplx<R>* data, int64_t S, int64_t inner,
                          int64_t outer, int64_t outer_stride, int n_in, int n_out, int mode, const int* omap,
                          int oper) {
    constexpr int W = strided_w_v<R, NN, (V & 7)>();
    constexpr int TPL = NN / PlanOf<R, NN, P>::E;
    constexpr long TILE = (long)sizeof(cplx<R>) * W * NN;
    constexpr bool PP = 2 * TILE <= 200 * 1024;
    const size_t smem = PP ? 2 * TILE : TILE;
    auto kern = k_fft_strided_reg<R, NN, W, P, PP>;
    static const bool once = (line_set_smem(kern, smem), true);
    (void)once;
    dim3 grid((unsigned)((inner + W - 1) / W), (unsigned)outer);
    line_launch(c, kern, grid, dim3(W * TPL), smem, data, S, inner, outer_stride, n_in, n_out, mode, c.ph, tw, omap,
                oper);
  }

  template <int NN, int D>
  static void row(const LineCtx<R>& c, const Tw<R>& tw, const RowArgs<R>& a, int blocks) {
    constexpr int RPB = row_rpb_reg_v<R, NN, V>();
    constexpr int NT = RPB * (NN / PlanOf<R, NN, P>::E);
    constexpr long TILE = (long)sizeof(cplx<R>) * D * RPB * (NN + NN / 16);  // padded lines (RegRowIx)
    if constexpr (NT > 1024 || 2 * TILE > 200 * 1024) {
      fail(SBEC_ERR_UNSUPPORTED, "row pass tile too large for this line length");
    } else {
      const size_t smem = 2 * TILE;
      auto kern = k_row_pass_reg<R, NN, D, RPB, P, true>;
      static const bool once = (line_set_smem(kern, smem), true);
      (void)once;
      line_launch(c, kern, dim3((unsigned)blocks), dim3(NT), smem, a, c.st, c.ph, tw);
    }
  }

  template <int NN>
  static void row_n(const LineCtx<R>& c, const Tw<R>& tw, int D, const RowArgs<R>& a, int blocks) {
    switch (D) {
      case 1: row<NN, 1>(c, tw, a, blocks); break;
      case 3: row<NN, 3>(c, tw, a, blocks); break;
      case 5: row<NN, 5>(c, tw, a, blocks); break;
      default: fail(SBEC_ERR_UNSUPPORTED, "fused path needs D in {1,3,5}");
    }
  }
};

template <typename R, int V>
void RegKernels<R, V>::fft_strided(const LineCtx<R>& c, const Tw<R>& tw, int n, cplx<R>* data, int64_t S,
                                   int64_t inner, int64_t outer, int64_t outer_stride, int n_in, int n_out, int mode,
                                   const int* omap, int oper) {
  switch (n) {
#define SBEC_REG_STRIDED(NN)                                                                                  \
  case NN:                                                                                                    \
    RegImpl<R, V>::template fft_strided<NN>(c, tw, data, S, inner, outer, outer_stride, n_in, n_out, mode, omap, \
                                            oper);                                                            \
    return;
    SBEC_REG_STRIDED(32)
    SBEC_REG_STRIDED(64)
    SBEC_REG_STRIDED(128)
    SBEC_REG_STRIDED(256)
    SBEC_REG_STRIDED(512)
    SBEC_REG_STRIDED(1024)
#undef SBEC_REG_STRIDED
    default: fail(SBEC_ERR_UNSUPPORTED, "unsupported strided FFT length " + std::to_string(n) + " for line variant " +
                                            std::to_string(V));
  }
}

template <typename R, int V>
void RegKernels<R, V>::row(const LineCtx<R>& c, const Tw<R>& tw, int n, int D, const RowArgs<R>& a, int blocks) {
  switch (n) {
    case 32: RegImpl<R, V>::template row_n<32>(c, tw, D, a, blocks); return;
    case 64: RegImpl<R, V>::template row_n<64>(c, tw, D, a, blocks); return;
    case 128: RegImpl<R, V>::template row_n<128>(c, tw, D, a, blocks); return;
    case 256: RegImpl<R, V>::template row_n<256>(c, tw, D, a, blocks); return;
    case 512: RegImpl<R, V>::template row_n<512>(c, tw, D, a, blocks); return;
    case 1024: RegImpl<R, V>::template row_n<1024>(c, tw, D, a, blocks); return;
    case 2048: RegImpl<R, V>::template row_n<2048>(c, tw, D, a, blocks); return;
    case 4096: RegImpl<R, V>::template row_n<4096>(c, tw, D, a, blocks); return;
    default: fail(SBEC_ERR_UNSUPPORTED, "unsupported row length " + std::to_string(n) + " for row variant " +
                                            std::to_string(V));
  }
}

}  // namespace sbec
