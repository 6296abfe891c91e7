// Shared-memory Stockham FFT for power-of-two line lengths 2..4096.
//
// A tile of lines sits in shared memory; element (line l, index i) lives at
// s[i*SI + l*SL].  Each line is transformed by TPL = N/E threads, E being the
// largest radix of the line's plan, so every thread holds E values in registers
// per stage.  A stage of radix RAD reads its inputs at stride N/RAD, applies the
// Stockham twiddles W_N^{r*(j mod Ns)*N/(Ns*RAD)}, runs a register DFT of size
// RAD and writes to the autosorted positions (j div Ns)*Ns*RAD + (j mod Ns) + r*Ns.
// Output is in natural order; forward is unnormalised (FFTW's fft!), the inverse
// is the unnormalised conjugate transform (normalisation is folded elsewhere).
#pragma once

#include "sbec_common.cuh"

namespace sbec {

// cos and sin of 2*pi*j/16, j = 0..7 (constants of the unit circle).
__device__ __forceinline__ double cos16(int j) {
  constexpr double c[8] = {1.0,
                           0.92387953251128675613,
                           0.70710678118654752440,
                           0.38268343236508977173,
                           0.0,
                           -0.38268343236508977173,
                           -0.70710678118654752440,
                           -0.92387953251128675613};
  return c[j];
}
__device__ __forceinline__ double sin16(int j) {
  constexpr double s[8] = {0.0,
                           0.38268343236508977173,
                           0.70710678118654752440,
                           0.92387953251128675613,
                           1.0,
                           0.92387953251128675613,
                           0.70710678118654752440,
                           0.38268343236508977173};
  return s[j];
}

// x * exp(SIGN * 2*pi*i*k/N) for compile-time N <= 16 and (after unrolling) constant k < N/2.
template <typename R, int N, int SIGN>
__device__ __forceinline__ cplx<R> twmul(cplx<R> x, int k) {
  const int j = k * (16 / N);
  if (j == 0) return x;
  if (j == 4) return SIGN < 0 ? mul_mi(x) : mul_i(x);
  if (j == 2 || j == 6) {
    R a, b;  // x * (±1 + SIGN i) before the 1/sqrt(2) scale
    if (j == 2) {
      a = SIGN < 0 ? x.x + x.y : x.x - x.y;
      b = SIGN < 0 ? x.y - x.x : x.y + x.x;
    } else {
      a = SIGN < 0 ? x.y - x.x : -(x.x + x.y);
      b = SIGN < 0 ? -(x.x + x.y) : x.x - x.y;
    }
    if constexpr (sizeof(R) == 4) {
      const float hh = 0.70710677f, hl = 1.2101617e-08f;  // 1/sqrt(2) = hh + hl
      // single rounding of a*hh + a*hl: the tail must not be added after the head is rounded
      return mk<R>(fmaf(a, hh, a * hl), fmaf(b, hh, b * hl));
    } else {
      const R h = (R)0.70710678118654752440;
      return mk<R>(h * a, h * b);
    }
  }
  if constexpr (sizeof(R) == 4) {
    const double c = cos16(j), sn = SIGN * sin16(j);
    const float2 wh = mk<float>((float)c, (float)sn);
    const float2 wl = mk<float>((float)(c - (double)wh.x), (float)(sn - (double)wh.y));
    return cmul_comp(x, wh, wl);
  } else {
    const cplx<R> w = mk<R>((R)cos16(j), (R)(SIGN * sin16(j)));
    return x * w;
  }
}

// In-register DFT of compile-time size N (1, 2, 4, 8, 16) by radix-2 decimation in time.
template <typename R, int N, int SIGN>
__device__ __forceinline__ void dft(cplx<R>* v) {
  if constexpr (N == 1) {
    return;
  } else if constexpr (N == 2) {
    const cplx<R> a = v[0], b = v[1];
    v[0] = a + b;
    v[1] = a - b;
  } else {
    cplx<R> e[N / 2], o[N / 2];
#pragma unroll
    for (int k = 0; k < N / 2; ++k) {
      e[k] = v[2 * k];
      o[k] = v[2 * k + 1];
    }
    dft<R, N / 2, SIGN>(e);
    dft<R, N / 2, SIGN>(o);
#pragma unroll
    for (int k = 0; k < N / 2; ++k) {
      const cplx<R> t = twmul<R, N, SIGN>(o[k], k);
      v[k] = e[k] + t;
      v[k + N / 2] = e[k] - t;
    }
  }
}

// Twiddles and butterflies of one Stockham stage on the values v a thread loaded
// (butterfly b holds v[b*RAD .. b*RAD+RAD-1], read at j + r*N/RAD, j = t + b*TPL).
template <typename R, int N, int E, int RAD, int SIGN>
__device__ __forceinline__ void fft_stage_math(int t, int Ns, const Tw<R>& tw, cplx<R> (&v)[E]) {
  constexpr int TPL = N / E;
  constexpr int NBT = E / RAD;
#pragma unroll
  for (int b = 0; b < NBT; ++b) {
    const int j = t + b * TPL;
    const int jm = j & (Ns - 1);
    if (Ns > 1) {
      const int step = jm * (N / (Ns * RAD));
#pragma unroll
      for (int r = 1; r < RAD; ++r) v[b * RAD + r] = tw_mul<R>(v[b * RAD + r], tw, r * step, SIGN > 0);
    }
    dft<R, RAD, SIGN>(&v[b * RAD]);
  }
}

// Twiddle, butterfly and store of one Stockham stage for the values v a thread loaded.
template <typename R, int N, int E, int RAD, int SIGN>
__device__ __forceinline__ void fft_stage_store(cplx<R>* s, int SI, int SL, int l, int t, int Ns, const Tw<R>& tw,
                                                cplx<R> (&v)[E]) {
  constexpr int TPL = N / E;
  constexpr int NBT = E / RAD;
  fft_stage_math<R, N, E, RAD, SIGN>(t, Ns, tw, v);
#pragma unroll
  for (int b = 0; b < NBT; ++b) {
    const int j = t + b * TPL;
    const int jm = j & (Ns - 1);
    const int base = (j - jm) * RAD + jm;
#pragma unroll
    for (int r = 0; r < RAD; ++r) s[(base + r * Ns) * SI + l * SL] = v[b * RAD + r];
  }
}

// One Stockham stage.  tw holds W_N^e = exp(-2*pi*i*e/N), e = 0..N-1 (forward sign).
// Threads with act == false (the spare threads of a block sized for a per-point
// stage) skip the work but reach the same two barriers as every other thread:
// __syncthreads is an aligned barrier, and a warp whose threads split between two
// barrier call sites never completes.
template <typename R, int N, int E, int RAD, int SIGN>
__device__ __forceinline__ void fft_stage(cplx<R>* s, int SI, int SL, int l, int t, int Ns, const Tw<R>& tw,
                                          bool act) {
  constexpr int TPL = N / E;
  constexpr int NBT = E / RAD;
  constexpr int STRIDE = N / RAD;
  cplx<R> v[E];
  if (act) {
#pragma unroll
    for (int b = 0; b < NBT; ++b) {
      const int j = t + b * TPL;
#pragma unroll
      for (int r = 0; r < RAD; ++r) v[b * RAD + r] = s[(j + r * STRIDE) * SI + l * SL];
    }
  }
  __syncthreads();
  if (act) fft_stage_store<R, N, E, RAD, SIGN>(s, SI, SL, l, t, Ns, tw, v);
  __syncthreads();
}

// One Stockham stage from src into a separate buffer dst: the loads of this stage
// cannot be overwritten by its own stores, so one barrier (after the stores) suffices.
template <typename R, int N, int E, int RAD, int SIGN>
__device__ __forceinline__ void fft_stage_pp(const cplx<R>* src, cplx<R>* dst, int SI, int SL, int l, int t, int Ns,
                                             const Tw<R>& tw, bool act) {
  constexpr int TPL = N / E;
  constexpr int NBT = E / RAD;
  constexpr int STRIDE = N / RAD;
  if (act) {
    cplx<R> v[E];
#pragma unroll
    for (int b = 0; b < NBT; ++b) {
      const int j = t + b * TPL;
#pragma unroll
      for (int r = 0; r < RAD; ++r) v[b * RAD + r] = src[(j + r * STRIDE) * SI + l * SL];
    }
    fft_stage_store<R, N, E, RAD, SIGN>(dst, SI, SL, l, t, Ns, tw, v);
  }
  __syncthreads();
}

// The stages alternating between buffers a and b; returns the buffer holding the result.
template <typename R, int N, int E, int SIGN, int RAD, int... REST>
__device__ __forceinline__ cplx<R>* run_stages_pp(cplx<R>* a, cplx<R>* b, int SI, int SL, int l, int t, int Ns,
                                                  const Tw<R>& tw, bool act) {
  fft_stage_pp<R, N, E, RAD, SIGN>(a, b, SI, SL, l, t, Ns, tw, act);
  if constexpr (sizeof...(REST) > 0)
    return run_stages_pp<R, N, E, SIGN, REST...>(b, a, SI, SL, l, t, Ns * RAD, tw, act);
  else
    return b;
}

template <typename R, int N, int E, int SIGN, int RAD, int... REST>
__device__ __forceinline__ void run_stages(cplx<R>* s, int SI, int SL, int l, int t, int Ns, const Tw<R>& tw,
                                           bool act) {
  fft_stage<R, N, E, RAD, SIGN>(s, SI, SL, l, t, Ns, tw, act);
  if constexpr (sizeof...(REST) > 0) run_stages<R, N, E, SIGN, REST...>(s, SI, SL, l, t, Ns * RAD, tw, act);
}

// ---- register-resident transforms (the D lines of one row per thread)
//
// Thread t of a line keeps the values at positions x = t + k*TPL (k < E, TPL = N/E) in u[k].
// Butterfly b of a radix-RAD Stockham stage reads positions j + r*N/RAD with j = t + b*TPL,
// i.e. slot k = b + r*(E/RAD) of u; the first stage (Ns = 1) can therefore take its inputs
// straight from u, and the last stage (Ns = N/RAD, where (j mod Ns) = j) writes its outputs
// to those same positions.  A transform thus starts from and ends in registers, with shared
// memory used only between its stages (one barrier per inner stage in the ping-pong form).
// Same twiddles, butterflies and order of operations as the tile transforms above, so the
// results are bit-identical to them.
template <int E, int RAD>
__host__ __device__ constexpr int reg_slot(int e) {
  return e / RAD + (e % RAD) * (E / RAD);
}

// Shared-memory index of element i of line l for the register-resident transforms.  Rows
// (RegRowIx): line after line, one complex of padding after every 16, which takes the 4-way
// bank conflicts out of the radix-4/8 Stockham stores (j*RAD + r, a stride of RAD elements
// across a half-warp) at 1/16 more shared memory.  Strided tiles (RegColIx): element (i, w)
// at i*W + w, as the tile form (consecutive threads are consecutive lines there).
struct RegRowIx {
  int line;  // N + N/16
  __device__ __forceinline__ int operator()(int i, int l) const { return l * line + i + (i >> 4); }
};
struct RegColIx {
  int W;
  __device__ __forceinline__ int operator()(int i, int l) const { return i * W + l; }
};

// Stores of one stage after fft_stage_math (the autosorted positions of fft_stage_store).
template <typename R, int N, int E, int RAD, typename Ix>
__device__ __forceinline__ void reg_stage_store(cplx<R>* dst, const Ix& ix, int l, int t, int Ns,
                                                const cplx<R> (&v)[E]) {
  constexpr int TPL = N / E;
  constexpr int NBT = E / RAD;
#pragma unroll
  for (int b = 0; b < NBT; ++b) {
    const int j = t + b * TPL;
    const int jm = j & (Ns - 1);
    const int base = (j - jm) * RAD + jm;
#pragma unroll
    for (int r = 0; r < RAD; ++r) dst[ix(base + r * Ns, l)] = v[b * RAD + r];
  }
}

// First stage: registers -> dst (lines l0 .. l0+D-1 of the tile).
template <typename R, int N, int E, int RAD, int SIGN, int D, typename Ix>
__device__ __forceinline__ void reg_stage_first(const cplx<R> (&u)[D][E], cplx<R>* dst, const Ix& ix, int l0, int t,
                                                const Tw<R>& tw) {
#pragma unroll
  for (int c = 0; c < D; ++c) {
    cplx<R> v[E];
#pragma unroll
    for (int e = 0; e < E; ++e) v[e] = u[c][reg_slot<E, RAD>(e)];
    fft_stage_math<R, N, E, RAD, SIGN>(t, 1, tw, v);
    reg_stage_store<R, N, E, RAD>(dst, ix, l0 + c, t, 1, v);
  }
}

template <typename R, int N, int E, int RAD, typename Ix>
__device__ __forceinline__ void reg_stage_load(const cplx<R>* src, const Ix& ix, int l, int t, cplx<R> (&v)[E]) {
  constexpr int TPL = N / E;
  constexpr int NBT = E / RAD;
  constexpr int STRIDE = N / RAD;
#pragma unroll
  for (int b = 0; b < NBT; ++b) {
#pragma unroll
    for (int r = 0; r < RAD; ++r) v[b * RAD + r] = src[ix(t + b * TPL + r * STRIDE, l)];
  }
}

// Stages after the first: inner stages through shared memory, the last one into registers.
// On entry cur holds the previous stage's output and every thread has passed the barrier
// after its stores; oth is free (ping-pong form).
template <typename R, int N, int E, int SIGN, bool PP, int D, typename Ix, int RAD, int... REST>
__device__ __forceinline__ void reg_stages(cplx<R> (&u)[D][E], cplx<R>*& cur, cplx<R>*& oth, const Ix& ix, int l0,
                                           int t, int Ns, const Tw<R>& tw) {
  if constexpr (sizeof...(REST) == 0) {
#pragma unroll
    for (int c = 0; c < D; ++c) {
      cplx<R> v[E];
      reg_stage_load<R, N, E, RAD>(cur, ix, l0 + c, t, v);
      fft_stage_math<R, N, E, RAD, SIGN>(t, Ns, tw, v);
#pragma unroll
      for (int e = 0; e < E; ++e) u[c][reg_slot<E, RAD>(e)] = v[e];
    }
  } else {
    if constexpr (PP) {
#pragma unroll
      for (int c = 0; c < D; ++c) {
        cplx<R> v[E];
        reg_stage_load<R, N, E, RAD>(cur, ix, l0 + c, t, v);
        fft_stage_math<R, N, E, RAD, SIGN>(t, Ns, tw, v);
        reg_stage_store<R, N, E, RAD>(oth, ix, l0 + c, t, Ns, v);
      }
      __syncthreads();
      cplx<R>* x = cur;
      cur = oth;
      oth = x;
    } else {
      cplx<R> v[D][E];
#pragma unroll
      for (int c = 0; c < D; ++c) reg_stage_load<R, N, E, RAD>(cur, ix, l0 + c, t, v[c]);
      __syncthreads();
#pragma unroll
      for (int c = 0; c < D; ++c) {
        fft_stage_math<R, N, E, RAD, SIGN>(t, Ns, tw, v[c]);
        reg_stage_store<R, N, E, RAD>(cur, ix, l0 + c, t, Ns, v[c]);
      }
      __syncthreads();
    }
    reg_stages<R, N, E, SIGN, PP, D, Ix, REST...>(u, cur, oth, ix, l0, t, Ns * RAD, tw);
  }
}

// A whole transform of the D lines held in u.  The first stage writes into oth (ping-pong
// form): cur may still be read by the last stage of a transform before.  The in-place
// form has one buffer and waits for those reads first.  On return the last stage has
// read cur and oth is free again.
template <typename R, int N, int E, int SIGN, bool PP, int D, typename Ix, int RAD0, int... REST>
__device__ __forceinline__ void reg_fft_run(cplx<R> (&u)[D][E], cplx<R>*& cur, cplx<R>*& oth, const Ix& ix, int l0,
                                            int t, const Tw<R>& tw) {
  static_assert(sizeof...(REST) >= 1, "register transforms need at least two stages");
  if constexpr (PP) {
    reg_stage_first<R, N, E, RAD0, SIGN, D>(u, oth, ix, l0, t, tw);
    __syncthreads();
    cplx<R>* x = cur;
    cur = oth;
    oth = x;
  } else {
    __syncthreads();
    reg_stage_first<R, N, E, RAD0, SIGN, D>(u, cur, ix, l0, t, tw);
    __syncthreads();
  }
  reg_stages<R, N, E, SIGN, PP, D, Ix, REST...>(u, cur, oth, ix, l0, t, RAD0, tw);
}

// Radix plans per line length: E = largest radix; stages run in the listed order.
// FP64 (FP64-throughput bound) uses radix-16 stages, which need the fewest
// twiddle multiplies; FP32 (latency / bandwidth bound) uses radix-4/8 stages so
// each line is spread over 4x more threads and the SMs hold more warps.
template <int N> struct FftPlan;
template <int N> struct FftPlan32;
#define SBEC_PLAN(STRUCT, NN, EE, ...)                                                          \
  template <> struct STRUCT<NN> {                                                                \
    static constexpr int E = EE;                                                                 \
    template <typename R, int SIGN>                                                              \
    static __device__ __forceinline__ void run(cplx<R>* s, int SI, int SL, int l, int t,        \
                                               const Tw<R>& tw, bool act) {                      \
      run_stages<R, NN, EE, SIGN, __VA_ARGS__>(s, SI, SL, l, t, 1, tw, act);                     \
    }                                                                                            \
    template <typename R, int SIGN>                                                              \
    static __device__ __forceinline__ cplx<R>* run_pp(cplx<R>* a, cplx<R>* b, int SI, int SL,   \
                                                      int l, int t, const Tw<R>& tw, bool act) { \
      return run_stages_pp<R, NN, EE, SIGN, __VA_ARGS__>(a, b, SI, SL, l, t, 1, tw, act);        \
    }                                                                                            \
    template <typename R, int SIGN, bool PP, int D, typename Ix>                                 \
    static __device__ __forceinline__ void run_reg(cplx<R> (&u)[D][EE], cplx<R>*& cur,          \
                                                   cplx<R>*& oth, const Ix& ix, int l0, int t,   \
                                                   const Tw<R>& tw) {                            \
      reg_fft_run<R, NN, EE, SIGN, PP, D, Ix, __VA_ARGS__>(u, cur, oth, ix, l0, t, tw);         \
    }                                                                                            \
  };
SBEC_PLAN(FftPlan, 2, 2, 2)
SBEC_PLAN(FftPlan, 4, 4, 4)
SBEC_PLAN(FftPlan, 8, 8, 8)
SBEC_PLAN(FftPlan, 16, 16, 16)
SBEC_PLAN(FftPlan, 32, 8, 8, 4)
SBEC_PLAN(FftPlan, 64, 8, 8, 8)
SBEC_PLAN(FftPlan, 128, 16, 16, 8)
SBEC_PLAN(FftPlan, 256, 16, 16, 16)
SBEC_PLAN(FftPlan, 512, 8, 8, 8, 8)
SBEC_PLAN(FftPlan, 1024, 16, 16, 8, 8)
SBEC_PLAN(FftPlan, 2048, 16, 16, 16, 8)
SBEC_PLAN(FftPlan, 4096, 16, 16, 16, 16)
SBEC_PLAN(FftPlan32, 2, 2, 2)
SBEC_PLAN(FftPlan32, 4, 4, 4)
SBEC_PLAN(FftPlan32, 8, 4, 4, 2)
SBEC_PLAN(FftPlan32, 16, 4, 4, 4)
SBEC_PLAN(FftPlan32, 32, 4, 4, 4, 2)
SBEC_PLAN(FftPlan32, 64, 4, 4, 4, 4)
SBEC_PLAN(FftPlan32, 128, 4, 4, 4, 4, 2)
SBEC_PLAN(FftPlan32, 256, 4, 4, 4, 4, 4)
SBEC_PLAN(FftPlan32, 512, 8, 8, 8, 8)
SBEC_PLAN(FftPlan32, 1024, 8, 8, 8, 4, 4)
SBEC_PLAN(FftPlan32, 2048, 8, 8, 8, 8, 4)
SBEC_PLAN(FftPlan32, 4096, 8, 8, 8, 8, 8)
#undef SBEC_PLAN

// Plan family P of a line kernel: 0 = the precision's default (radix-16 for FP64,
// radix-4/8 for FP32), 1 = the other one.  The autotuner picks per shape.
template <typename R, int N, int P>
struct PlanSel;
template <int N>
struct PlanSel<double, N, 0> {
  using type = FftPlan<N>;
};
template <int N>
struct PlanSel<double, N, 1> {
  using type = FftPlan32<N>;
};
template <int N>
struct PlanSel<float, N, 0> {
  using type = FftPlan32<N>;
};
template <int N>
struct PlanSel<float, N, 1> {
  using type = FftPlan<N>;
};
template <typename R, int N, int P = 0>
using PlanOf = typename PlanSel<R, N, P>::type;

// host-side mirror of PlanOf<R, N, P>::E
inline int plan_radix_host(bool fp32, int n, int P = 0) {
  const bool deep = fp32 ? (P == 1) : (P == 0);
  if (!deep) return n <= 4 ? n : (n <= 256 ? 4 : 8);
  switch (n) {
    case 32: case 64: case 512: return 8;
    case 2: case 4: case 8: return n;
    default: return 16;
  }
}

// Transform every line of a shared-memory tile (all threads of the block participate).
// Caller must __syncthreads() after filling the tile; the function ends synchronised.
template <typename R, int N, int SIGN, int P = 0>
__device__ __forceinline__ void fft_tile(cplx<R>* s, int SI, int SL, int l, int t, const Tw<R>& tw,
                                         bool act = true) {
  PlanOf<R, N, P>::template run<R, SIGN>(s, SI, SL, l, t, tw, act);
}

// Ping-pong form: the tile in a, the same-sized buffer b; returns the buffer holding the
// transform (a or b, by the parity of the stage count).  One barrier per stage.
template <typename R, int N, int SIGN, int P = 0>
__device__ __forceinline__ cplx<R>* fft_tile_pp(cplx<R>* a, cplx<R>* b, int SI, int SL, int l, int t, const Tw<R>& tw,
                                                bool act = true) {
  return PlanOf<R, N, P>::template run_pp<R, SIGN>(a, b, SI, SL, l, t, tw, act);
}

// The transform of the tile at cur: in place (PP false, two barriers per stage) or
// ping-pong through oth (PP true, one barrier per stage).  On return cur points at
// the result and oth at the other buffer.
template <typename R, int N, int SIGN, int P, bool PP>
__device__ __forceinline__ void fft_tile_sel(cplx<R>*& cur, cplx<R>*& oth, int SI, int SL, int l, int t,
                                             const Tw<R>& tw, bool act = true) {
  if constexpr (PP) {
    cplx<R>* r = fft_tile_pp<R, N, SIGN, P>(cur, oth, SI, SL, l, t, tw, act);
    if (r != cur) {
      oth = cur;
      cur = r;
    }
  } else {
    fft_tile<R, N, SIGN, P>(cur, SI, SL, l, t, tw, act);
  }
}

}  // namespace sbec
