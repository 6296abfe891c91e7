// Device kernels of the split-step engine, templated on the working real type R
// (double: the plain FP64 form; float: the FP32-bulk form).  Reductions always
// accumulate in double.
#pragma once

#include "sbec_common.cuh"
#include "sbec_fft.cuh"

namespace sbec {

// ---------------------------------------------------------------------------
// Kinetic phase tables
// ---------------------------------------------------------------------------
// exp(-i k^2 dt/2) (or exp(-k^2 dt/2) in imaginary time) factorises over axes:
// tab_a[m] = exp(-i k_a(m)^2 dt/2) with k_a(m) = fftfreq index * kmult_a
// (src/propagators.jl:1-7, 137-145).  The 1/prod(n) normalisation of the inverse
// FFT (FFTW ifft!) is folded into the axis-0 table.
struct PhaseTableArgs {
  int n[3];
  double kmult[3];
  double dt;
  double scale;
  int ndim;
  int itp;
};

template <typename R>
struct PhaseOut {
  cplx<R>* hi[3];
  cplx<R>* lo[3];
};

template <typename R>
__global__ void k_phase_tables(PhaseOut<R> out, PhaseTableArgs a) {
  const int axis = blockIdx.y;
  if (axis >= a.ndim) return;
  cplx<R>* tab = out.hi[axis];
  cplx<R>* tlo = out.lo[axis];
  const int n = a.n[axis];
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < n; m += gridDim.x * blockDim.x) {
    const int idx = m < (n + 1) / 2 ? m : m - n;
    const double k = (double)idx * a.kmult[axis];
    const double arg = -0.5 * (k * k) * a.dt;
    double re, im;
    if (a.itp) {
      re = exp(arg);
      im = 0.0;
    } else {
      sincos(arg, &im, &re);
    }
    if (axis == 0) {
      re *= a.scale;
      im *= a.scale;
    }
    const cplx<R> h = mk<R>((R)re, (R)im);
    if constexpr (sizeof(R) == 4) {
      tab[2 * m] = h;
      tab[2 * m + 1] = mk<R>((R)(re - (double)h.x), (R)(im - (double)h.y));
    } else {
      tab[m] = h;
    }
    (void)tlo;
  }
}

template <typename R>
struct PhaseRef {
  Tw<R> tab[3];
  int n[3];
  int ndim;
  R scale0;      // exact power-of-two scale folded into tab[0] (1/N)
  int unbiased;  // real-time FP32 tables: phase_mul's unbiased form
};

// The FP32 real-time kinetic factor of a 2-D / 3-D point: the per-axis factors
// scale_a (1 + c_a + i s_a) (tables: head and tail; scale 1/N on x, 1 elsewhere, both
// exact powers of two) are combined as (1 + C + iS) = prod_a (1 + c_a + i s_a) in the
// small quantities c_a, s_a (full relative precision for low k), and x is turned once:
// x/N + (x/N)(C + iS) with the addition rounded without bias (sr_add).
// (1 + C + iS) <- (1 + C + iS)(1 + c + is) for the table entry scale (1 + c + is).
__device__ __forceinline__ void kin_fold(float& C, float& Sn, const Tw<float>& t, int idx, float scale, float inv) {
  const float4 w4 = __ldg(reinterpret_cast<const float4*>(t.hi) + idx);
  const float c = __fmul_rn(__fadd_rn(__fsub_rn(w4.x, scale), w4.z), inv);
  const float sn = __fmul_rn(__fadd_rn(w4.y, w4.w), inv);
  const float nC = __fadd_rn(__fadd_rn(C, c), __fmaf_rn(C, c, __fmul_rn(-Sn, sn)));
  const float nS = __fadd_rn(__fadd_rn(Sn, sn), __fmaf_rn(Sn, c, __fmul_rn(C, sn)));
  C = nC;
  Sn = nS;
}

__device__ __forceinline__ float2 kinetic_rot(float2 x, const PhaseRef<float>& ph, int i0, int i1, int ilast) {
  float C = 0.0f, Sn = 0.0f;
  const float inv0 = 1.0f / ph.scale0;  // N: exact
  kin_fold(C, Sn, ph.tab[0], i0, ph.scale0, inv0);
  if (ph.ndim == 3) kin_fold(C, Sn, ph.tab[1], i1, 1.0f, 1.0f);
  kin_fold(C, Sn, ph.tab[ph.ndim - 1], ilast, 1.0f, 1.0f);
  const float2 xs = mk<float>(__fmul_rn(x.x, ph.scale0), __fmul_rn(x.y, ph.scale0));
  const float bx = __fmaf_rn(xs.x, C, __fmul_rn(-xs.y, Sn));
  const float by = __fmaf_rn(xs.y, C, __fmul_rn(xs.x, Sn));
  return mk<float>(sr_add(xs.x, bx, 0x85ebca6bu), sr_add(xs.y, by, 0xc2b2ae35u));
}

// The same rotation for any number of axes and a scale 1/N that need not be a power of
// two: the rounding error of x * scale0 (exact, from an fma) joins the small term, so the
// one rounded addition left is the unbiased one.
__device__ __forceinline__ float2 kinetic_rot_any(float2 x, const PhaseRef<float>& ph, int i0, int i1, int i2) {
  float C = 0.0f, Sn = 0.0f;
  kin_fold(C, Sn, ph.tab[0], i0, ph.scale0, __frcp_rn(ph.scale0));
  if (ph.ndim >= 2) kin_fold(C, Sn, ph.tab[1], i1, 1.0f, 1.0f);
  if (ph.ndim == 3) kin_fold(C, Sn, ph.tab[2], i2, 1.0f, 1.0f);
  const float2 xs = mk<float>(__fmul_rn(x.x, ph.scale0), __fmul_rn(x.y, ph.scale0));
  const float ex = __fmaf_rn(x.x, ph.scale0, -xs.x), ey = __fmaf_rn(x.y, ph.scale0, -xs.y);
  const float bx = __fadd_rn(__fmaf_rn(xs.x, C, __fmul_rn(-xs.y, Sn)), ex);
  const float by = __fadd_rn(__fmaf_rn(xs.y, C, __fmul_rn(xs.x, Sn)), ey);
  return mk<float>(sr_add(xs.x, bx, 0x85ebca6bu), sr_add(xs.y, by, 0xc2b2ae35u));
}

// ---------------------------------------------------------------------------
// Axes whose length n is not a power of two: Bluestein's identity
//   X_k = w_k sum_j (x_j w_j) conj(w_{k-j}),  w_j = exp(-+ i pi j^2 / n),
// a circular convolution of length M >= 2n - 1 (a power of two) done with the power-of-two
// line kernels: chirp and zero-pad (k_blue_pre), forward M-point FFT, multiply by the
// M-point FFT of the chirp (k_blue_mid), inverse M-point FFT, chirp, scale 1/M and keep the
// first n points (k_blue_post).  The lines of an axis with element stride `inner` (the product
// of the lower axis lengths) are laid out in the scratch as [outer][j][inner], so both the
// grid and the scratch are read and written with inner fastest (coalesced), and the M-point
// transforms run as strided lines of the same geometry (contiguous lines when inner = 1).
// ---------------------------------------------------------------------------
// The chirp and its spectrum are (head, tail) pairs in FP32 (cmul_comp: the factor to about
// 2^-48): a table that enters every transform with the same rounding would otherwise change
// the norm by the same amount at every step.
template <typename R>
__global__ void k_blue_pre(const cplx<R>* __restrict__ src, cplx<R>* __restrict__ scr, int n, int M, int64_t inner,
                           int64_t total, const cplx<R>* __restrict__ chirp, const cplx<R>* __restrict__ chirp_lo) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i_in = q % inner, r = q / inner;
    const int j = (int)(r % M);
    const int64_t i_out = r / M;
    scr[q] = j < n ? cmul_comp(src[i_in + (int64_t)j * inner + i_out * inner * n], __ldg(chirp + j),
                               __ldg(chirp_lo + j))
                   : mk<R>(0, 0);
  }
}

template <typename R>
__global__ void k_blue_mid(cplx<R>* __restrict__ scr, int M, int64_t inner, int64_t total,
                           const cplx<R>* __restrict__ bhat, const cplx<R>* __restrict__ bhat_lo) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t m = (q / inner) % M;
    scr[q] = cmul_comp(scr[q], __ldg(bhat + m), __ldg(bhat_lo + m));
  }
}

template <typename R>
__global__ void k_blue_post(const cplx<R>* __restrict__ scr, cplx<R>* __restrict__ dst, int n, int M, int64_t inner,
                            int64_t total, const cplx<R>* __restrict__ chirp, const cplx<R>* __restrict__ chirp_lo,
                            R inv_m) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i_in = q % inner, r = q / inner;
    const int k = (int)(r % n);
    const int64_t i_out = r / n;
    const cplx<R> v = cmul_comp(scr[(i_out * M + k) * inner + i_in], __ldg(chirp + k), __ldg(chirp_lo + k));
    dst[i_in + (int64_t)k * inner + i_out * inner * n] = inv_m * v;  // 1/M: a power of two
  }
}

// The kinetic phase of a grid with a non-power-of-two axis, applied between the forward and
// inverse transforms of all axes: the product of the per-axis table entries (1/N folded
// into the x table), one compensated product per axis in FP32; in FP32 real time the
// unbiased single rotation of kinetic_rot_any.
template <typename R>
__global__ void k_kinetic_apply(cplx<R>* __restrict__ buf, int64_t N, int64_t total, PhaseRef<R> ph) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = q % N;
    const int i0 = (int)(p % ph.n[0]);
    const int64_t r = p / ph.n[0];
    if constexpr (sizeof(R) == 4) {
      if (ph.unbiased) {
        buf[q] = kinetic_rot_any(buf[q], ph, i0, ph.ndim >= 2 ? (int)(r % ph.n[1]) : 0,
                                 ph.ndim == 3 ? (int)(r / ph.n[1]) : 0);
        continue;
      }
    }
    cplx<R> v = phase_mul<R>(buf[q], ph.tab[0], i0, ph.scale0, 0);
    if (ph.ndim >= 2) v = phase_mul<R>(v, ph.tab[1], (int)(r % ph.n[1]), (R)1, 0);
    if (ph.ndim == 3) v = phase_mul<R>(v, ph.tab[2], (int)(r / ph.n[1]), (R)1, 0);
    buf[q] = v;
  }
}

// A load of line data: plain (may be served by L1), or CG: through L2 only, for data
// that other blocks of the same launch wrote (the persistent segment kernel).
template <bool CG, typename T>
__device__ __forceinline__ T ld_line(const T* p) {
  if constexpr (CG) return __ldcg(p);
  else return *p;
}

// ---------------------------------------------------------------------------
// FFT along x (contiguous lines).  mode 0: forward, 1: inverse,
// 2: forward, x phase (1-D kinetic step), inverse.
// PP: the stages ping-pong between two tiles of shared memory (one barrier each).
// ---------------------------------------------------------------------------
template <typename R, int N, int LPB, int P = 0, bool PP = false>
__global__ void __launch_bounds__(LPB * (N / PlanOf<R, N, P>::E))
k_fft_x(cplx<R>* __restrict__ data, int64_t n_lines, int mode, PhaseRef<R> ph, Tw<R> tw) {
  pdl_wait();
  constexpr int TPL = N / PlanOf<R, N, P>::E;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<R>* s = reinterpret_cast<cplx<R>*>(smem_raw);
  cplx<R>* s2 = s + LPB * N;
  const int tid = threadIdx.x;
  const int64_t line0 = (int64_t)blockIdx.x * LPB;
  const int nl = (int)min((int64_t)LPB, n_lines - line0);
  cplx<R>* g = data + line0 * N;
  for (int f = tid; f < LPB * N; f += blockDim.x) s[f] = (f < nl * N) ? g[f] : mk<R>(0, 0);
  __syncthreads();
  const int t = tid % TPL, l = tid / TPL;
  if (mode == 1) {
    fft_tile_sel<R, N, +1, P, PP>(s, s2, 1, N, l, t, tw);
  } else {
    fft_tile_sel<R, N, -1, P, PP>(s, s2, 1, N, l, t, tw);
    if (mode == 2) {
      for (int f = tid; f < LPB * N; f += blockDim.x) s[f] = phase_mul<R>(s[f], ph.tab[0], f % N, ph.scale0, ph.unbiased);
      __syncthreads();
      fft_tile_sel<R, N, +1, P, PP>(s, s2, 1, N, l, t, tw);
    }
  }
  pdl_trigger();
  for (int f = tid; f < nl * N; f += blockDim.x) g[f] = s[f];
}

// ---------------------------------------------------------------------------
// FFT along a strided axis.  Line (o, w) starts at o*outer_stride + i0 + w and
// has elements at stride S.  Loads only i < n_in (zero beyond), stores only
// i < n_out (pruned transforms of the zero-padded DDI grid).
// mode 0 forward, 1 inverse, 2 forward, x phase, inverse (last axis of the
// kinetic step; the line's lower-axis coordinates come from i0 + w).
// PP: the stages ping-pong between two tiles of shared memory (one barrier each).
// ---------------------------------------------------------------------------
// The work of one block: W lines starting at inner index i0 of outer line o.  CG: load
// the lines through L2 only (the persistent segment kernel reads data other blocks wrote
// during the same launch).  trig: signal dependent launches before the final stores.
template <typename R, int N, int W, int P, bool PP, bool CG>
__device__ __forceinline__ void fft_strided_block(cplx<R>* __restrict__ data, int64_t S, int64_t inner,
                                                  int64_t outer_stride, int n_in, int n_out, int mode,
                                                  const PhaseRef<R>& ph, const Tw<R>& tw, int64_t i0, int64_t o,
                                                  unsigned char* smem_raw, bool trig) {
  constexpr int TPL = N / PlanOf<R, N, P>::E;
  cplx<R>* s = reinterpret_cast<cplx<R>*>(smem_raw);
  cplx<R>* s2 = s + W * N;
  __shared__ cplx<R> inner_ph[W];
  __shared__ int inner_idx[W][2];
  const int tid = threadIdx.x;
  const int nw = (int)min((int64_t)W, inner - i0);
  cplx<R>* g = data + o * outer_stride + i0;
  for (int f = tid; f < W * N; f += blockDim.x) {
    const int i = f / W, w = f % W;
    s[f] = (i < n_in && w < nw) ? ld_line<CG>(g + (int64_t)i * S + w) : mk<R>(0, 0);
  }
  if (mode == 2 && tid < W) {
    // lower-axis factors of the kinetic phase for this line
    int64_t pos = i0 + tid;
    cplx<R> f = mk<R>(1, 0);
    inner_idx[tid][1] = -1;
    for (int a = 0; a < ph.ndim - 1; ++a) {
      const int ia = (int)(pos % ph.n[a]);
      pos /= ph.n[a];
      inner_idx[tid][a] = ia;
      f = f * __ldg(ph.tab[a].hi + ia);
    }
    inner_ph[tid] = f;
  }
  __syncthreads();
  const int w = tid % W, t = tid / W;
  if (mode == 1) {
    fft_tile_sel<R, N, +1, P, PP>(s, s2, W, 1, w, t, tw);
  } else {
    fft_tile_sel<R, N, -1, P, PP>(s, s2, W, 1, w, t, tw);
    if (mode == 2) {
      const Tw<R> last = ph.tab[ph.ndim - 1];
      for (int f = tid; f < W * N; f += blockDim.x) {
        const int i = f / W, ww = f % W;
        if constexpr (sizeof(R) == 8) {
          s[f] = s[f] * (inner_ph[ww] * __ldg(last.hi + i));
        } else if (ph.unbiased) {
          // FP32 real time: all axis factors as one rotation, applied with one unbiased rounding
          s[f] = kinetic_rot(s[f], ph, inner_idx[ww][0], ph.ndim == 3 ? inner_idx[ww][1] : 0, i);
        } else {
          // FP32 imaginary time: one compensated product per axis factor
          cplx<R> v = phase_mul<R>(s[f], ph.tab[0], inner_idx[ww][0], ph.scale0, 0);
          if (ph.ndim == 3) v = phase_mul<R>(v, ph.tab[1], inner_idx[ww][1], (R)1, 0);
          s[f] = phase_mul<R>(v, last, i, (R)1, 0);
        }
      }
      __syncthreads();
      fft_tile_sel<R, N, +1, P, PP>(s, s2, W, 1, w, t, tw);
    }
  }
  if (trig) pdl_trigger();
  for (int f = tid; f < W * N; f += blockDim.x) {
    const int i = f / W, ww = f % W;
    if (i < n_out && ww < nw) g[(int64_t)i * S + ww] = s[f];
  }
}

template <typename R, int N, int W, int P = 0, bool PP = false>
__global__ void __launch_bounds__(W * (N / PlanOf<R, N, P>::E))
k_fft_strided(cplx<R>* __restrict__ data, int64_t S, int64_t inner, int64_t outer_stride, int n_in,
              int n_out, int mode, PhaseRef<R> ph, Tw<R> tw, const int* __restrict__ omap, int oper) {
  pdl_wait();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int64_t o = omap ? (int64_t)omap[blockIdx.y / oper] * oper + blockIdx.y % oper : (int64_t)blockIdx.y;
  fft_strided_block<R, N, W, P, PP, false>(data, S, inner, outer_stride, n_in, n_out, mode, ph, tw,
                                           (int64_t)blockIdx.x * W, o, smem_raw, true);
}

// Register-resident form of k_fft_strided (same modes, pruning, arithmetic and results): thread
// (w, t) of a tile of W lines holds elements i = t + k*TPL (k < E) of line w in registers, loads
// them from and stores them to global memory directly (the same coalescing as the tile
// loads: W consecutive elements per row), and in mode 2 multiplies the kinetic phase on the
// registers between the forward and the inverse transform; shared memory (element (i, w) at
// i*W + w) carries only the transforms' inner stages.
template <typename R, int N, int W, int P, bool PP>
__global__ void __launch_bounds__(W*(N / PlanOf<R, N, P>::E))
k_fft_strided_reg(cplx<R>* __restrict__ data, int64_t S, int64_t inner, int64_t outer_stride, int n_in, int n_out,
                  int mode, PhaseRef<R> ph, Tw<R> tw, const int* __restrict__ omap, int oper) {
  constexpr int E = PlanOf<R, N, P>::E;
  constexpr int TPL = N / E;
  pdl_wait();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<R>* cur = reinterpret_cast<cplx<R>*>(smem_raw);
  cplx<R>* oth = cur + W * N;
  const RegColIx ix{W};
  const int64_t o = omap ? (int64_t)omap[blockIdx.y / oper] * oper + blockIdx.y % oper : (int64_t)blockIdx.y;
  const int64_t i0 = (int64_t)blockIdx.x * W;
  const int tid = threadIdx.x;
  const int w = tid % W, t = tid / W;
  const bool live = i0 + w < inner;
  cplx<R>* g = data + o * outer_stride + i0;
  cplx<R> u[1][E];
#pragma unroll
  for (int k = 0; k < E; ++k) {
    const int i = t + k * TPL;
    u[0][k] = (live && i < n_in) ? g[(int64_t)i * S + w] : mk<R>(0, 0);
  }
  if (mode == 1) {
    PlanOf<R, N, P>::template run_reg<R, +1, PP, 1>(u, cur, oth, ix, w, t, tw);
  } else {
    PlanOf<R, N, P>::template run_reg<R, -1, PP, 1>(u, cur, oth, ix, w, t, tw);
    if (mode == 2) {
      // lower-axis coordinates and factors of the kinetic phase for this line
      int64_t pos = i0 + w;
      cplx<R> f = mk<R>(1, 0);
      int idx0 = 0, idx1 = 0;
      if (ph.ndim >= 2) {
        idx0 = (int)(pos % ph.n[0]);
        pos /= ph.n[0];
        f = f * __ldg(ph.tab[0].hi + idx0);
      }
      if (ph.ndim == 3) {
        idx1 = (int)(pos % ph.n[1]);
        f = f * __ldg(ph.tab[1].hi + idx1);
      }
      const Tw<R> last = ph.tab[ph.ndim - 1];
#pragma unroll
      for (int k = 0; k < E; ++k) {
        const int i = t + k * TPL;
        if constexpr (sizeof(R) == 8) {
          u[0][k] = u[0][k] * (f * __ldg(last.hi + i));
        } else if (ph.unbiased) {
          u[0][k] = kinetic_rot(u[0][k], ph, idx0, idx1, i);
        } else {
          cplx<R> v = phase_mul<R>(u[0][k], ph.tab[0], idx0, ph.scale0, 0);
          if (ph.ndim == 3) v = phase_mul<R>(v, ph.tab[1], idx1, (R)1, 0);
          u[0][k] = phase_mul<R>(v, last, i, (R)1, 0);
        }
      }
      PlanOf<R, N, P>::template run_reg<R, +1, PP, 1>(u, cur, oth, ix, w, t, tw);
    }
  }
  pdl_trigger();
  if (live) {
#pragma unroll
    for (int k = 0; k < E; ++k) {
      const int i = t + k * TPL;
      if (i < n_out) g[(int64_t)i * S + w] = u[0][k];
    }
  }
}

// ---------------------------------------------------------------------------
// Dipolar convolution (src/ddi.jl:108-136, src/ddi_padded.jl:55-85).
// Real spin-density fields live on the simulation grid (nx, ny, nz); the
// convolution grid has (Mx, My, Mz) = n (periodic) or 2n (zero padded).  The
// half spectrum (Mx/2+1, My, nz) of each of the 3 fields is stored with the
// z-extent pruned to nz: z >= nz is zero before the z transform and never read
// after it.  Φ̂ = C' (k (k·F̂)/k² - F̂/3), Q(0) = 0, computed on the fly from k
// (src/ddi.jl:7-40); the secular variant keeps only the zz part.
// ---------------------------------------------------------------------------
struct DdiGeom {
  int nx, ny, nz;      // simulation grid (active corner)
  int Mx, My, Mz;      // convolution grid
  int Hx;              // Mx/2 + 1
  int64_t field_stride;  // complex elements per field in the spectrum buffer (Hx*My*nz)
  double kmx, kmy, kmz;  // k multipliers of the convolution grid
  double C;            // C_dd / (Mx*My*Mz): contraction scale incl. inverse normalisation
  int secular;
  int ndim;
};

// FP32 form: Q from k in FP32 (the FP64 pipe, ~1/64 of the FP32 rate here, had bound the
// last-axis DDI pass); Q_ab = k_a k_b / k^2 - delta_ab/3 to FP32 rounding.
__device__ __forceinline__ void ddi_contract_f32(float2& fx, float2& fy, float2& fz, float kx, float ky, float kz,
                                                 const DdiGeom& g) {
  const float k2 = kx * kx + ky * ky + kz * kz;
  if (k2 == 0.0f) {
    fx = fy = fz = make_float2(0.f, 0.f);
    return;
  }
  const float inv = 1.0f / k2;
  const float C = (float)g.C;
  if (g.secular) {
    const float qzz = kz * kz * inv - (1.0f / 3.0f);
    const float qxx = -0.5f * qzz;
    fx = (C * qxx) * fx;
    fy = (C * qxx) * fy;
    fz = (C * qzz) * fz;
    return;
  }
  const float qxx = kx * kx * inv - (1.0f / 3.0f), qyy = ky * ky * inv - (1.0f / 3.0f),
              qzz = kz * kz * inv - (1.0f / 3.0f);
  const float qxy = kx * ky * inv, qxz = kx * kz * inv, qyz = ky * kz * inv;
  const float2 px = C * (qxx * fx + qxy * fy + qxz * fz);
  const float2 py = C * (qxy * fx + qyy * fy + qyz * fz);
  const float2 pz = C * (qxz * fx + qyz * fy + qzz * fz);
  fx = px;
  fy = py;
  fz = pz;
}

template <typename R>
__device__ __forceinline__ void ddi_contract(cplx<R>& fx, cplx<R>& fy, cplx<R>& fz, double kx, double ky,
                                             double kz, const DdiGeom& g) {
  if constexpr (sizeof(R) == 4) {
    ddi_contract_f32(fx, fy, fz, (float)kx, (float)ky, (float)kz, g);
    return;
  }
  const double k2 = kx * kx + ky * ky + kz * kz;
  if (k2 == 0.0) {
    fx = fy = fz = mk<R>(0, 0);
    return;
  }
  const double inv = 1.0 / k2;
  if (g.secular) {
    const R qzz = (R)(kz * kz * inv - 1.0 / 3.0);
    const R qxx = -qzz / (R)2;
    const R C = (R)g.C;
    fx = (C * qxx) * fx;
    fy = (C * qxx) * fy;
    fz = (C * qzz) * fz;
    return;
  }
  const R qxx = (R)(kx * kx * inv - 1.0 / 3.0), qyy = (R)(ky * ky * inv - 1.0 / 3.0),
          qzz = (R)(kz * kz * inv - 1.0 / 3.0);
  const R qxy = (R)(kx * ky * inv), qxz = (R)(kx * kz * inv), qyz = (R)(ky * kz * inv);
  const R C = (R)g.C;
  const cplx<R> px = C * (qxx * fx + qxy * fy + qxz * fz);
  const cplx<R> py = C * (qxy * fx + qyy * fy + qyz * fz);
  const cplx<R> pz = C * (qxz * fx + qyz * fy + qzz * fz);
  fx = px;
  fy = py;
  fz = pz;
}

__device__ __forceinline__ int freq_index(int m, int M) { return m < (M + 1) / 2 ? m : m - M; }

// C2R pre-processing for a half spectrum X[0..MH]: returns 2 Z_k with
// Z_k = E_k + i O_k, E_k = (X_k + conj X_{MH-k})/2, O_k = (X_k - conj X_{MH-k}) W^{-k}/2.
// Like FFTW's / pocketfft's c2r, only the real parts of the DC and Nyquist
// entries are used (their imaginary parts are dropped); the DDI spectrum at the
// x-Nyquist plane is not Hermitian in (ky, kz) because Q_xy, Q_xz are odd there.
template <typename R>
__device__ __forceinline__ cplx<R> c2r_pre(const cplx<R>* X, int k, int MH, const Tw<R>& tw_full) {
  cplx<R> Xk = X[k];
  cplx<R> Xc = conj(X[MH - k]);
  if (k == 0) {
    Xk.y = 0;
    Xc.y = 0;
  }
  return (Xk + Xc) + mul_i(tw_mul<R>(Xk - Xc, tw_full, k, true));
}

// R2C along x of the 3 real fields, via a complex FFT of length MH = Mx/2 on
// z[j] = f[2j] + i f[2j+1] followed by the split X[k] = E_k + W_Mx^k O_k.
// Rows (y < ny, z < nz) only; output row (y, z) at spectrum row y + My*z.
// tw_half: W_MH table; tw_full: W_Mx table.  For 1-D (ndim == 1) the kernel
// also contracts and returns to real space (the x axis is the last axis).
template <typename R, int MH, int LPB>
__global__ void __launch_bounds__(3 * LPB * (MH / PlanOf<R, MH>::E))
k_ddi_r2c_x(const R* __restrict__ f3, int64_t field_n, cplx<R>* __restrict__ spec, DdiGeom g,
            R* __restrict__ phi3, Tw<R> tw_half, Tw<R> tw_full) {
  constexpr int TPL = MH / PlanOf<R, MH>::E;
  constexpr int NL = 3 * LPB;  // lines in the tile: field-major
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<R>* s = reinterpret_cast<cplx<R>*>(smem_raw);   // NL * MH
  cplx<R>* xs = s + NL * MH;                            // NL * (MH + 1) split output
  const int tid = threadIdx.x;
  const int64_t n_rows = (int64_t)g.ny * g.nz;
  const int64_t row0 = (int64_t)blockIdx.x * LPB;
  const int nr = (int)min((int64_t)LPB, n_rows - row0);
  for (int f = tid; f < NL * MH; f += blockDim.x) {
    const int line = f / MH, j = f % MH;
    const int fld = line / LPB, r = line % LPB;
    cplx<R> v = mk<R>(0, 0);
    if (r < nr) {
      const R* src = f3 + fld * field_n + (row0 + r) * g.nx;
      const int x0 = 2 * j, x1 = 2 * j + 1;
      v.x = x0 < g.nx ? src[x0] : (R)0;
      v.y = x1 < g.nx ? src[x1] : (R)0;
    }
    s[f] = v;
  }
  __syncthreads();
  const int t = tid % TPL, l = tid / TPL;
  fft_tile<R, MH, -1>(s, 1, MH, l, t, tw_half);
  // split into the half spectrum X[0..MH]
  for (int f = tid; f < NL * (MH + 1); f += blockDim.x) {
    const int line = f / (MH + 1), k = f % (MH + 1);
    const cplx<R> Zk = s[line * MH + (k % MH)];
    const cplx<R> Zc = conj(s[line * MH + ((MH - k) % MH)]);
    const cplx<R> E = (R)0.5 * (Zk + Zc);
    const cplx<R> O = (R)0.5 * mul_mi(Zk - Zc);
    xs[f] = (k == MH) ? (E - O) : E + tw_mul<R>(O, tw_full, k % (2 * MH), false);
  }
  __syncthreads();
  if (g.ndim > 1) {
    for (int f = tid; f < NL * (MH + 1); f += blockDim.x) {
      const int line = f / (MH + 1), k = f % (MH + 1);
      const int fld = line / LPB, r = line % LPB;
      if (r >= nr) continue;
      const int64_t row = row0 + r;
      const int64_t y = row % g.ny, z = row / g.ny;
      spec[fld * g.field_stride + (y + (int64_t)g.My * z) * g.Hx + k] = xs[f];
    }
    return;
  }
  // 1-D: contract at kx and go back to real space in the same tile.
  for (int f = tid; f < LPB * (MH + 1); f += blockDim.x) {
    const int r = f / (MH + 1), k = f % (MH + 1);
    cplx<R>& ax = xs[(0 * LPB + r) * (MH + 1) + k];
    cplx<R>& ay = xs[(1 * LPB + r) * (MH + 1) + k];
    cplx<R>& az = xs[(2 * LPB + r) * (MH + 1) + k];
    ddi_contract<R>(ax, ay, az, (double)k * g.kmx, 0.0, 0.0, g);
  }
  __syncthreads();
  // C2R: Z_k = (X_k + conj X_{MH-k}) + i (X_k - conj X_{MH-k}) W_Mx^{-k}, k < MH
  for (int f = tid; f < NL * MH; f += blockDim.x) {
    const int line = f / MH, k = f % MH;
    s[f] = c2r_pre(xs + line * (MH + 1), k, MH, tw_full);
  }
  __syncthreads();
  fft_tile<R, MH, +1>(s, 1, MH, l, t, tw_half);
  for (int f = tid; f < NL * MH; f += blockDim.x) {
    const int line = f / MH, j = f % MH;
    const int fld = line / LPB, r = line % LPB;
    if (r >= nr) continue;
    R* dst = phi3 + fld * field_n + (row0 + r) * g.nx;
    const int x0 = 2 * j, x1 = 2 * j + 1;
    if (x0 < g.nx) dst[x0] = s[f].x;
    if (x1 < g.nx) dst[x1] = s[f].y;
  }
}

// C2R along x of the 3 fields (rows y < ny, z < nz), keeping x < nx.
template <typename R, int MH, int LPB>
__global__ void __launch_bounds__(3 * LPB * (MH / PlanOf<R, MH>::E))
k_ddi_c2r_x(const cplx<R>* __restrict__ spec, DdiGeom g, R* __restrict__ phi3, int64_t field_n,
            Tw<R> tw_half, Tw<R> tw_full) {
  constexpr int TPL = MH / PlanOf<R, MH>::E;
  constexpr int NL = 3 * LPB;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<R>* s = reinterpret_cast<cplx<R>*>(smem_raw);
  cplx<R>* xs = s + NL * MH;
  const int tid = threadIdx.x;
  const int64_t n_rows = (int64_t)g.ny * g.nz;
  const int64_t row0 = (int64_t)blockIdx.x * LPB;
  const int nr = (int)min((int64_t)LPB, n_rows - row0);
  for (int f = tid; f < NL * (MH + 1); f += blockDim.x) {
    const int line = f / (MH + 1), k = f % (MH + 1);
    const int fld = line / LPB, r = line % LPB;
    cplx<R> v = mk<R>(0, 0);
    if (r < nr) {
      const int64_t row = row0 + r;
      const int64_t y = row % g.ny, z = row / g.ny;
      v = spec[fld * g.field_stride + (y + (int64_t)g.My * z) * g.Hx + k];
    }
    xs[f] = v;
  }
  __syncthreads();
  for (int f = tid; f < NL * MH; f += blockDim.x) {
    const int line = f / MH, k = f % MH;
    s[f] = c2r_pre(xs + line * (MH + 1), k, MH, tw_full);
  }
  __syncthreads();
  const int t = tid % TPL, l = tid / TPL;
  fft_tile<R, MH, +1>(s, 1, MH, l, t, tw_half);
  for (int f = tid; f < NL * MH; f += blockDim.x) {
    const int line = f / MH, j = f % MH;
    const int fld = line / LPB, r = line % LPB;
    if (r >= nr) continue;
    R* dst = phi3 + fld * field_n + (row0 + r) * g.nx;
    const int x0 = 2 * j, x1 = 2 * j + 1;
    if (x0 < g.nx) dst[x0] = s[f].x;
    if (x1 < g.nx) dst[x1] = s[f].y;
  }
}

// Last axis of the DDI convolution (y in 2-D, z in 3-D): forward transform of
// the 3 fields' lines (first n_in entries, zero beyond), contraction, inverse
// transform, store of the first n_out entries.  Lines: inner index = position
// in the lower axes of the spectrum (kx [, ky]), stride S between elements.
template <typename R, int M, int W>
__global__ void __launch_bounds__(3 * W * (M / PlanOf<R, M>::E))
k_ddi_last(cplx<R>* __restrict__ spec, DdiGeom g, int64_t S, int64_t inner, int n_in, int n_out, Tw<R> tw) {
  constexpr int TPL = M / PlanOf<R, M>::E;
  constexpr int NL = 3 * W;   // line index = fld*W + w
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<R>* s = reinterpret_cast<cplx<R>*>(smem_raw);   // element (line, i) at s[i*NL + line]
  const int tid = threadIdx.x;
  const int64_t i0 = (int64_t)blockIdx.x * W;
  const int nw = (int)min((int64_t)W, inner - i0);
  for (int f = tid; f < NL * M; f += blockDim.x) {
    const int i = f / NL, line = f % NL;
    const int fld = line / W, w = line % W;
    s[f] = (i < n_in && w < nw) ? spec[fld * g.field_stride + i0 + w + (int64_t)i * S] : mk<R>(0, 0);
  }
  __syncthreads();
  const int line = tid % NL, t = tid / NL;
  fft_tile<R, M, -1>(s, NL, 1, line, t, tw);
  for (int f = tid; f < W * M; f += blockDim.x) {
    const int i = f / W, w = f % W;
    const int64_t pos = i0 + w;
    cplx<R>& ax = s[i * NL + 0 * W + w];
    cplx<R>& ay = s[i * NL + 1 * W + w];
    cplx<R>& az = s[i * NL + 2 * W + w];
    if constexpr (sizeof(R) == 4) {
      // frequency indices times the k multipliers, all in FP32 (the FP64 pipe is slow here)
      float kx, ky, kz;
      if (g.ndim == 2) {
        kx = (float)pos * (float)g.kmx;
        ky = (float)freq_index(i, M) * (float)g.kmy;
        kz = 0.0f;
      } else {
        const int p = (int)pos;  // < Hx * My, which fits an int
        kx = (float)(p % g.Hx) * (float)g.kmx;
        ky = (float)freq_index(p / g.Hx, g.My) * (float)g.kmy;
        kz = (float)freq_index(i, M) * (float)g.kmz;
      }
      ddi_contract_f32(ax, ay, az, kx, ky, kz, g);
    } else {
      double kx, ky, kz;
      if (g.ndim == 2) {
        kx = (double)pos * g.kmx;
        ky = (double)freq_index(i, M) * g.kmy;
        kz = 0.0;
      } else {
        kx = (double)(pos % g.Hx) * g.kmx;
        ky = (double)freq_index((int)(pos / g.Hx), g.My) * g.kmy;
        kz = (double)freq_index(i, M) * g.kmz;
      }
      ddi_contract<R>(ax, ay, az, kx, ky, kz, g);
    }
  }
  __syncthreads();
  fft_tile<R, M, +1>(s, NL, 1, line, t, tw);
  for (int f = tid; f < NL * M; f += blockDim.x) {
    const int i = f / NL, ln = f % NL;
    const int fld = ln / W, w = ln % W;
    if (i < n_out && w < nw) spec[fld * g.field_stride + i0 + w + (int64_t)i * S] = s[f];
  }
}

// ---------------------------------------------------------------------------
// Pointwise potential stage (src/split_step.jl:48-133 minus the FFT work):
//   [diag(tau_d)] [rot_a: spin mixing(tau_s)] [DDI rotation(tau_ddi)]
//   [rot_b: spin mixing(tau_s)] [diag(tau_d)] [spin density out]
// ---------------------------------------------------------------------------
template <typename R>
struct SpinTabs {
  cplx<R> V[kMaxD * kMaxD];    // Fy eigenvectors (columns), ascending eigenvalues
  cplx<R> Vt[kMaxD * kMaxD];   // adjoint
  R fp[kMaxD];                 // f+(m_c) = sqrt(F(F+1) - m_c(m_c+1)), c >= 1
  R m[kMaxD];                  // m_c = F - c
};

// Raman coupling H_R(r) = delta Fz + (Omega/2)(e^{ik.r} F+ + e^{-ik.r} F-) (src/raman.jl:1-31).
// With F+- = Fx +- iFy this is b(r)·F, b = (Omega cos k.r, -Omega sin k.r, delta), so its
// exponential is a spin rotation about b(r) (the reference exponentiates the same Hermitian
// matrix by eigen-decomposition, src/spinor_utils.jl:27-38).  Grid coordinates
// x_d = x0_d + i_d dx_d (src/grid.jl:2-7), point index p = i0 + n0 (i1 + n1 i2).
struct RamanGeom {
  double omega, delta;
  double k[3], x0[3], dx[3];
  int n0, n1;
};

__device__ __forceinline__ void raman_field(const RamanGeom& g, int64_t p, double& bx, double& by, double& bz) {
  const int64_t i0 = p % g.n0, r = p / g.n0;
  const int64_t i1 = r % g.n1, i2 = r / g.n1;
  const double kr = g.k[0] * (g.x0[0] + (double)i0 * g.dx[0]) + g.k[1] * (g.x0[1] + (double)i1 * g.dx[1]) +
                    g.k[2] * (g.x0[2] + (double)i2 * g.dx[2]);
  double sn, cs;
  sincos(kr, &sn, &cs);
  bx = g.omega * cs;
  by = -g.omega * sn;
  bz = g.delta;
}

template <typename R>
struct PotArgs {
  cplx<R>* psi;
  int64_t N;
  const R* V;
  const R* phi;                // DDI potential fields (3*N) or null
  R* spin_out;                 // spin density output (3*N) or null
  int pre_diag, rot_a, ddi_rot, rot_b, post_diag;
  int nem_a, nem_b;            // singlet-pair (nematic) steps after rot_a / before rot_b
  int itp;
  R tau_d, tau_s, tau_ddi;
  R c0, c1, c_lhy, c2;
  cplx<R> zee[kMaxD];          // per-component Zeeman factor for diag(tau_d)
  cplx<R> zee_lo[kMaxD];       // FP32 real time: (cos theta - 1, sin theta) of the factor e^{i theta}
  // Raman rotation exp(-i tau_r b(r)·F) after nem_a (raman_a) / before nem_b (raman_b)
  int raman_a, raman_b;
  R tau_r;
  RamanGeom rg;
};

// Upper bound of the Taylor sub-steps of one exponential (rotation or tensor step):
// legitimate states need a few; an overflowed state (|phi| or n infinite) gets this
// many and finishes with a non-finite result instead of looping for 2^31 sub-steps.
constexpr int kMaxSub = 4096;

// sin x and cos x - 1 in FP32.  For |x| <= 1/2 (the usual case: the phase angles of
// one split step are small) both come from their Taylor series, summed by Horner's
// rule in x^2 through the x^9 and x^10 terms (the first omitted term is below 3e-11
// of the result at |x| = 1/2); cos x - 1 is formed directly, so it keeps full relative
// precision for small x.  Larger angles use one sincosf of x/2:
// sin x = 2 sin(x/2) cos(x/2), cos x - 1 = -2 sin^2(x/2).
__device__ __forceinline__ void sin_cosm1(float x, float& sn, float& cm1) {
  if (fabsf(x) <= 0.5f) {
    const float x2 = x * x;
    const float ps = fmaf(x2, fmaf(x2, fmaf(x2, 1.0f / 362880.0f, -1.0f / 5040.0f), 1.0f / 120.0f), -1.0f / 6.0f);
    sn = fmaf(x * x2, ps, x);
    const float pc = fmaf(x2, fmaf(x2, fmaf(x2, fmaf(x2, -1.0f / 3628800.0f, 1.0f / 40320.0f), -1.0f / 720.0f),
                                   1.0f / 24.0f),
                          -0.5f);
    cm1 = x2 * pc;
  } else {
    float sh, ch;
    sincosf(0.5f * x, &sh, &ch);
    sn = 2.0f * sh * ch;
    cm1 = -2.0f * sh * sh;
  }
}

// z (1 + cm1 - i sn) = z + z (cm1 - i sn) for a small FP32 rotation: the whole
// correction (radial cm1 z and tangential -i sn z) is formed first and added with one
// rounding.  Left to FMA contraction the radial part is added last, in a rounding of
// its own, and is dropped whenever it is below half an ulp (|x| below ~2.4e-4, the trap
// centre) while the tangential part survives; the final addition is rounded without
// bias (sr_add).  The _rn intrinsics are not contracted.
__device__ __forceinline__ float2 rot_small(float2 z, float cm1, float sn) {
  const float bx = __fmaf_rn(z.x, cm1, __fmul_rn(z.y, sn));
  const float by = __fmaf_rn(z.y, cm1, __fmul_rn(-z.x, sn));
  return make_float2(sr_add(z.x, bx, 0x9e3779b9u), sr_add(z.y, by, 0x7f4a7c15u));
}

// z e^{-i phi} e^{i theta} (the potential phase and a Zeeman phase) as one rotation with one
// unbiased addition: (cm1, sn) = (cos phi - 1, sin phi), zcs = (cos theta - 1, sin theta).
// Turning z by the Zeeman factor in a separate rounded product would drop the radial part
// of the small rotation (below half an ulp) at every call and |z| would grow.
__device__ __forceinline__ float2 rot_small_zee(float2 z, float cm1, float sn, float2 zcs) {
  const float C = __fadd_rn(__fadd_rn(cm1, zcs.x), __fmaf_rn(cm1, zcs.x, __fmul_rn(sn, zcs.y)));
  const float S = __fadd_rn(__fsub_rn(zcs.y, sn), __fmaf_rn(cm1, zcs.y, __fmul_rn(-sn, zcs.x)));
  return rot_small(z, C, -S);
}

// u + (a A + b B) with the correction formed in full before the single addition to u
// (same reason as rot_small; a, b real coefficients, A, B complex).
__device__ __forceinline__ float2 add_corr(float2 u, float a, float2 A, float b, float2 B) {
  const float cx = __fmaf_rn(b, B.x, __fmul_rn(a, A.x));
  const float cy = __fmaf_rn(b, B.y, __fmul_rn(a, A.y));
  return make_float2(__fadd_rn(u.x, cx), __fadd_rn(u.y, cy));
}

// sinh x and cosh x - 1 in FP32 (the imaginary-time spin rotation): Taylor series
// through the x^9 / x^10 terms for |x| <= 1/2, as in sin_cosm1 (cosh x - 1 then keeps
// full relative precision, where coshf(x) - 1 cancels), otherwise from one expf.
__device__ __forceinline__ void sinh_coshm1(float x, float& sh, float& chm1) {
  if (fabsf(x) <= 0.5f) {
    const float x2 = x * x;
    const float ps = fmaf(x2, fmaf(x2, fmaf(x2, 1.0f / 362880.0f, 1.0f / 5040.0f), 1.0f / 120.0f), 1.0f / 6.0f);
    sh = fmaf(x * x2, ps, x);
    const float pc = fmaf(x2, fmaf(x2, fmaf(x2, fmaf(x2, 1.0f / 3628800.0f, 1.0f / 40320.0f), 1.0f / 720.0f),
                                   1.0f / 24.0f),
                          0.5f);
    chm1 = x2 * pc;
  } else {
    const float e = expf(x), ei = 1.0f / e;
    sh = 0.5f * (e - ei);
    chm1 = 0.5f * (e + ei) - 1.0f;
  }
}

// psi_c *= exp(-i Veff tau) * zee_c  (real time) or exp(-Veff tau) * zee_c (imaginary time),
// src/propagators.jl:95-116.  FP64 keeps the reference's product order; FP32 applies
// the potential phase as psi + psi*(cos x - 1, -sin x) with cos x - 1 from sin_cosm1:
// for the small angles of the trap centre cosf(x) rounds to 1 while sinf(x) does not,
// and a plain product would change |psi| systematically every step.
template <typename R, int D>
__device__ __forceinline__ void diag_apply(cplx<R> (&v)[D], R veff, R tau, int itp, const cplx<R>* zee,
                                           const cplx<R>* zee_lo) {
  if (itp) {
    const R e = exp(-veff * tau);
#pragma unroll
    for (int c = 0; c < D; ++c) {
      if constexpr (sizeof(R) == 8) v[c] = v[c] * (mk<R>(e, (R)0) * zee[c]);
      else v[c] = v[c] * (e * zee[c].x);  // imaginary-time Zeeman factors are real; renormalised each step
    }
    return;
  }
  if constexpr (sizeof(R) == 8) {
    const cplx<R> base = cis_(-veff * tau);
#pragma unroll
    for (int c = 0; c < D; ++c) v[c] = v[c] * (base * zee[c]);
  } else {
    float sn, cm1;
    sin_cosm1(veff * tau, sn, cm1);
#pragma unroll
    for (int c = 0; c < D; ++c) v[c] = rot_small_zee(v[c], cm1, sn, zee_lo[c]);
  }
}

template <typename R, int D>
__device__ __forceinline__ void diag_point(cplx<R> (&v)[D], R Vp, const PotArgs<R>& a, R c0) {
  R n = 0;
#pragma unroll
  for (int c = 0; c < D; ++c) n += abs2(v[c]);
  R Vint = c0 * n;
  if (a.c_lhy != (R)0) Vint += a.c_lhy * n * sqrt(n);
  diag_apply<R, D>(v, Vp + Vint, a.tau_d, a.itp, a.zee, a.zee_lo);
}

// <F> components from the raising operator (src/observables.jl:61-86).
template <typename R, int D>
__device__ __forceinline__ void spin_vector(const cplx<R> (&v)[D], const SpinTabs<R>& st, R& fx, R& fy,
                                            R& fz) {
  R z = 0, re = 0, im = 0;
#pragma unroll
  for (int c = 0; c < D; ++c) z += st.m[c] * abs2(v[c]);
#pragma unroll
  for (int c = 1; c < D; ++c) {
    const cplx<R> p = cmulc(v[c - 1], v[c]);
    re += st.fp[c] * p.x;
    im += st.fp[c] * p.y;
  }
  fx = re;
  fy = im;
  fz = z;
}

// (n·F) v with n = (nx, ny, nz): tridiagonal in the m basis.
template <typename R, int D>
__device__ __forceinline__ void nF_apply(const cplx<R> (&v)[D], R nx, R ny, R nz, const SpinTabs<R>& st,
                                         cplx<R> (&out)[D]) {
  const cplx<R> nm = mk<R>(nx * (R)0.5, -ny * (R)0.5);  // (nx - i ny)/2 multiplies F+
  const cplx<R> np = mk<R>(nx * (R)0.5, ny * (R)0.5);   // (nx + i ny)/2 multiplies F-
#pragma unroll
  for (int c = 0; c < D; ++c) {
    cplx<R> r = (nz * st.m[c]) * v[c];
    if (c + 1 < D) r += nm * (st.fp[c + 1] * v[c + 1]);
    if (c >= 1) r += np * (st.fp[c] * v[c - 1]);
    out[c] = r;
  }
}

// FP32 spin-1 rotation in Cartesian components.  With X = (v_-1 - v_+1, -i(v_+1 + v_-1),
// sqrt2 v_0) (sqrt2 times the Cartesian spinor), <F> = (Im(X_y* X_z), Im(X_z* X_x),
// Im(X_x* X_y)) and exp(-i th n·F) rotates Re X and Im X about n:
// X + sin th (n x X) + (cos th - 1)(X - n (n·X)); in imaginary time
// exp(-th n·F) X = X - i sinh th (n x X) + (cosh th - 1)(X - n (n·X)).  The m = 0
// component is kept unscaled (w = v_0, X_z = sqrt2 w) so the rounded sqrt2 only enters
// the correction terms; a scale in and out would change |v_0| by the same factor every
// call.  Same operator as the m-basis form below, with about half the arithmetic.
__device__ __forceinline__ void rodrigues_cart(float2 (&v)[3], float c1, float tau, int itp) {
  constexpr float s2 = 1.41421356237f, r2 = 0.70710678118f;
  const float2 Ux = v[2] - v[0];
  const float2 Uy = mul_mi(v[0] + v[2]);
  const float2 w = v[1];
  const float fx = s2 * (Uy.x * w.y - Uy.y * w.x);
  const float fy = s2 * (w.x * Ux.y - w.y * Ux.x);
  const float fz = Ux.x * Uy.y - Ux.y * Uy.x;
  const float f2 = fx * fx + fy * fy + fz * fz;
  if (!(f2 > 1e-37f)) return;  // |<F>| below ~1e-19 rotates by less than an ulp
  const float inv = rsqrtf(f2);
  const float nx = fx * inv, ny = fy * inv, nz = fz * inv;
  const float th = c1 * (f2 * inv) * tau;
  const float2 nX = nx * Ux + ny * Uy + (s2 * nz) * w;  // n·X
  const float2 cx = (s2 * ny) * w - nz * Uy;            // (n x X)_x
  const float2 cy = nz * Ux - (s2 * nx) * w;            // (n x X)_y
  const float2 czs = r2 * (nx * Uy - ny * Ux);          // (n x X)_z / sqrt2
  const float2 px = Ux - nx * nX, py = Uy - ny * nX, pw = w - (r2 * nz) * nX;  // X - n (n·X)
  float2 X, Y, W;
  if (itp) {
    float sh, chm1;
    sinh_coshm1(th, sh, chm1);
    X = Ux + mul_mi(sh * cx) + chm1 * px;
    Y = Uy + mul_mi(sh * cy) + chm1 * py;
    W = w + mul_mi(sh * czs) + chm1 * pw;
  } else {
    float sn, cm1;
    sin_cosm1(th, sn, cm1);
    X = add_corr(Ux, sn, cx, cm1, px);
    Y = add_corr(Uy, sn, cy, cm1, py);
    W = add_corr(w, sn, czs, cm1, pw);
  }
  const float2 iY = mul_i(Y);
  v[0] = 0.5f * (iY - X);
  v[1] = W;
  v[2] = 0.5f * (iY + X);
}

// Spin-1 Rodrigues rotation exp(-i theta n·F) (src/spin_mixing.jl:71-98).
template <typename R, int D>
__device__ __forceinline__ void rodrigues_point(cplx<R> (&v)[D], R c1, R tau, int itp, const SpinTabs<R>& st) {
  if constexpr (sizeof(R) == 4 && D == 3) {
    rodrigues_cart(v, c1, tau, itp);
    return;
  }
  R fx, fy, fz;
  spin_vector<R, D>(v, st, fx, fy, fz);
  R fm, inv;
  if constexpr (sizeof(R) == 8) {
    fm = sqrt(fx * fx + fy * fy + fz * fz);
    if (fm < (R)1e-30) return;
    inv = (R)1 / fm;
  } else {
    // |<F>| below ~1e-19 (|<F>|^2 under the FP32 normal range) rotates by less than an ulp
    const float f2 = fx * fx + fy * fy + fz * fz;
    if (!(f2 > 1e-37f)) return;
    inv = rsqrtf(f2);
    fm = f2 * inv;
  }
  cplx<R> w[D], w2[D];
  nF_apply<R, D>(v, fx * inv, fy * inv, fz * inv, st, w);
  nF_apply<R, D>(w, fx * inv, fy * inv, fz * inv, st, w2);
  const R th = c1 * fm * tau;
  if (itp) {
    R sh, chm1;
    if constexpr (sizeof(R) == 8) {
      sh = sinh(th);
      chm1 = cosh(th) - (R)1;
    } else {
      sinh_coshm1(th, sh, chm1);
    }
#pragma unroll
    for (int c = 0; c < D; ++c) v[c] = v[c] - sh * w[c] + chm1 * w2[c];
  } else {
    R sn, cm1;  // sin th and cos th - 1 (without cancellation)
    if constexpr (sizeof(R) == 8) {
      sn = sin(th);
      const R sh = sin(th * (R)0.5);
      cm1 = (R)-2 * sh * sh;
    } else {
      sin_cosm1(th, sn, cm1);
    }
#pragma unroll
    for (int c = 0; c < D; ++c) v[c] = v[c] + mul_mi(sn * w[c]) + cm1 * w2[c];
  }
}

// Euler-angle rotation exp(-i dt phi·F) (src/spinor_utils.jl:82-166).
template <typename R, int D>
__device__ __forceinline__ void euler_point(cplx<R> (&v)[D], R px, R py, R pz, R dt, int itp,
                                            const SpinTabs<R>& st) {
  constexpr int F = (D - 1) / 2;
  const R pm = sqrt(px * px + py * py + pz * pz);
  if (pm * fabs(dt) < (R)1e-14) return;
  R cz = pz / pm;
  cz = cz < (R)-1 ? (R)-1 : (cz > (R)1 ? (R)1 : cz);
  const R beta = acos(cz);
  const R alpha = atan2(py, px);
  const R theta = pm * dt;
  const cplx<R> z_neg_alpha = cis_(-alpha);
  const cplx<R> z_beta = cis_(beta);
  const cplx<R> rz_phase = cis_((R)F * alpha);
  const cplx<R> ry_phase = cis_(-(R)F * beta);
  cplx<R> w[D];
  cplx<R> phase = rz_phase;
#pragma unroll
  for (int c = 0; c < D; ++c) {
    v[c] = phase * v[c];
    phase = phase * z_neg_alpha;
  }
  phase = ry_phase;
#pragma unroll
  for (int i = 0; i < D; ++i) {
    cplx<R> s = mk<R>(0, 0);
#pragma unroll
    for (int j = 0; j < D; ++j) s += st.Vt[i * D + j] * v[j];
    w[i] = phase * s;
    phase = phase * z_beta;
  }
#pragma unroll
  for (int i = 0; i < D; ++i) {
    cplx<R> s = mk<R>(0, 0);
#pragma unroll
    for (int j = 0; j < D; ++j) s += st.V[i * D + j] * w[j];
    v[i] = s;
  }
  if (itp) {
    R dz_r = exp(-(R)F * theta);
    const R dz_step = exp(theta);
#pragma unroll
    for (int c = 0; c < D; ++c) {
      v[c] = v[c] * dz_r;
      dz_r = dz_r * dz_step;
    }
  } else {
    cplx<R> dz_phase = cis_(-(R)F * theta);
    const cplx<R> z_theta = cis_(theta);
#pragma unroll
    for (int c = 0; c < D; ++c) {
      v[c] = v[c] * dz_phase;
      dz_phase = dz_phase * z_theta;
    }
  }
  phase = conj(ry_phase);
  const cplx<R> z_neg_beta = conj(z_beta);
#pragma unroll
  for (int i = 0; i < D; ++i) {
    cplx<R> s = mk<R>(0, 0);
#pragma unroll
    for (int j = 0; j < D; ++j) s += st.Vt[i * D + j] * v[j];
    w[i] = phase * s;
    phase = phase * z_neg_beta;
  }
  phase = conj(rz_phase);
  const cplx<R> z_alpha = conj(z_neg_alpha);
#pragma unroll
  for (int i = 0; i < D; ++i) {
    cplx<R> s = mk<R>(0, 0);
#pragma unroll
    for (int j = 0; j < D; ++j) s += st.V[i * D + j] * w[j];
    v[i] = phase * s;
    phase = phase * z_alpha;
  }
}

// exp(-i tau phi·F) v (or exp(-tau phi·F) v in imaginary time) by a Taylor series
// of the tridiagonal phi·F, with sub-steps so each has ||tau phi·F|| <= 1/2 and the
// series cut once the bound of the next term is below eps.  The series is summed by
// Horner's scheme, v + (X/1)(v + (X/2)(v + ...)): adding the terms largest-first drops
// every term below half an ulp of the running sum, a truncation whose norm error has
// one sign (about -1e-7 per unit rotation angle in FP32), while the nested form adds
// each correction to a value of its own size.  Used by the FP32 form
// in place of the Euler-angle phases, whose FP32 recurrences carry a systematic
// magnitude error; the operator is the same exp(-i dt phi·F) as
// src/spinor_utils.jl:82-166 and the skip threshold |phi||dt| < 1e-14 is kept.
template <typename R, int D>
__device__ __forceinline__ void rotate_taylor(cplx<R> (&v)[D], R px, R py, R pz, R tau, int itp,
                                              const SpinTabs<R>& st, float eps) {
  constexpr int F = (D - 1) / 2;
  const R pm = sqrt(px * px + py * py + pz * pz);
  if (pm * fabs(tau) < (R)1e-14) return;
  const float bound = (float)(pm * fabs(tau)) * (float)F;
  // at most kMaxSub sub-steps: a non-finite state must not turn into an endless loop
  const int nsub = bound > 0.5f ? (bound < 0.5f * kMaxSub ? (int)ceilf(bound / 0.5f) : kMaxSub) : 1;
  const float xs = bound / (float)nsub;
  int K = 1;
  {
    float term = xs;
    while (K < 30 && term >= eps) {
      ++K;
      term *= xs / (float)K;
    }
  }
  const R dt = tau / (R)nsub;
  for (int sub = 0; sub < nsub; ++sub) {
    cplx<R> y[D];
#pragma unroll
    for (int c = 0; c < D; ++c) y[c] = v[c];
    for (int k = K; k >= 1; --k) {
      cplx<R> t[D];
      nF_apply<R, D>(y, px, py, pz, st, t);
      const R f = dt / (R)k;
      bool done_k = false;
      if constexpr (sizeof(R) == 4) {
        if (k == 1 && !itp) {
          // the last addition v + (whole correction) rounded without bias: for the small
          // angles of one step, round-to-nearest keeps a near-axis value outside the circle
          // (the radial part of the correction is below half an ulp) and |v| grows every call
#pragma unroll
          for (int c = 0; c < D; ++c) {
            const cplx<R> corr = mul_mi(f * t[c]);
            y[c] = mk<R>(sr_add(v[c].x, corr.x, 0x27d4eb2fu + 0x165667b1u * c),
                         sr_add(v[c].y, corr.y, 0x9e3779b1u + 0x85ebca77u * c));
          }
          done_k = true;
        }
      }
      if (!done_k) {
#pragma unroll
        for (int c = 0; c < D; ++c) y[c] = v[c] + (itp ? (-f) * t[c] : mul_mi(f * t[c]));
      }
    }
#pragma unroll
    for (int c = 0; c < D; ++c) v[c] = y[c];
  }
}

// Spin rotation used by the DDI step and general-D spin mixing: the reference's
// Euler-angle form in FP64, the Taylor form in FP32.
template <typename R, int D>
__device__ __forceinline__ void spin_rotate(cplx<R> (&v)[D], R px, R py, R pz, R tau, int itp,
                                            const SpinTabs<R>& st) {
  if constexpr (sizeof(R) == 8) euler_point<R, D>(v, px, py, pz, tau, itp, st);
  else rotate_taylor<R, D>(v, px, py, pz, tau, itp, st, 1e-13f);
}

// Spin mixing exp(-i c1 tau <F>·F) (src/spin_mixing.jl:1-66).
template <typename R, int D>
__device__ __forceinline__ void spin_mixing_point(cplx<R> (&v)[D], R c1, R tau, int itp, const SpinTabs<R>& st) {
  if constexpr (D == 3) {
    rodrigues_point<R, D>(v, c1, tau, itp, st);
  } else if constexpr (D > 1) {
    R fx, fy, fz;
    spin_vector<R, D>(v, st, fx, fy, fz);
    spin_rotate<R, D>(v, c1 * fx, c1 * fy, c1 * fz, tau, itp, st);
  }
}

// Singlet-pair (nematic) step (src/nematic.jl:53-119): A00 = sum_c (-1)^c psi_c psi_(D-1-c)
// / sqrt(D) from the state before the step (component c has m = F - c, so (-1)^(F-m) =
// (-1)^c); each (m, -m) pair, and m = 0 with itself, is turned by the exact solution of
// i d psi_m/dt = V psi*_(-m) with V = c2 A00 (-1)^c / sqrt(D):
//   real time  psi_m <- cos(|V| tau) psi_m - i (V/|V|) sin(|V| tau) psi*_(-m)
//   imaginary  psi_m <- cosh(|V| tau) psi_m - (V/|V|) sinh(|V| tau) psi*_(-m)
// pairs with |V| < 1e-30 (and every pair when |c2| < 1e-30) are left as they are.  FP32
// forms the rotation as psi + ((cos - 1) psi + ...) with cos - 1 kept to full precision.
// Kept out of line: the potential stages call it only when c2 is set, and inlining it
// would enlarge every row pass.
template <typename R, int D>
__device__ __noinline__ void nematic_point(cplx<R> (&v)[D], R c2, R tau, int itp) {
  if (!(fabs(c2) >= (R)1e-30)) return;
  const R isd = (R)(1.0 / sqrt((double)D));
  cplx<R> A = mk<R>(0, 0);
#pragma unroll
  for (int c = 0; c < D; ++c) {
    const cplx<R> pr = v[c] * v[D - 1 - c];
    A = (c & 1) ? A - pr : A + pr;
  }
  const cplx<R> Vb = (c2 * isd * isd) * A;
#pragma unroll
  for (int c = 0; c <= (D - 1) / 2; ++c) {
    const int cp = D - 1 - c;
    const cplx<R> V = (c & 1) ? mk<R>(-Vb.x, -Vb.y) : Vb;
    const R absV = sqrt(V.x * V.x + V.y * V.y);
    if (!(absV >= (R)1e-30)) continue;
    const cplx<R> ph = mk<R>(V.x / absV, V.y / absV);
    const R x = absV * tau;
    R cm1, sn;  // cos - 1 and -i sin (real time) or cosh - 1 and -sinh (imaginary time)
    cplx<R> b;  // coefficient of conj(psi_pair)
    if constexpr (sizeof(R) == 4) {
      if (itp) sinh_coshm1(x, sn, cm1);
      else sin_cosm1(x, sn, cm1);
    } else {
      if (itp) {
        sn = sinh(x);
        cm1 = cosh(x) - 1.0;
      } else {
        sincos(x, &sn, &cm1);
        cm1 -= 1.0;
      }
    }
    b = itp ? mk<R>(-ph.x * sn, -ph.y * sn) : mk<R>(ph.y * sn, -ph.x * sn);  // -ph sn | -i ph sn
    const cplx<R> vm = v[c], vn = v[cp];
    if constexpr (sizeof(R) == 8) {
      const R ca = cm1 + (R)1;
      v[c] = ca * vm + b * conj(vn);
      if (cp != c) v[cp] = ca * vn + b * conj(vm);
    } else {
      v[c] = vm + (cm1 * vm + b * conj(vn));
      if (cp != c) v[cp] = vn + (cm1 * vn + b * conj(vm));
    }
  }
}

template <typename R, int D>
__global__ void __launch_bounds__(256) k_potential(PotArgs<R> a, SpinTabs<R> st) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.N) return;
  cplx<R> v[D];
#pragma unroll
  for (int c = 0; c < D; ++c) v[c] = a.psi[c * a.N + p];
  const R Vp = a.V[p];
  if (a.pre_diag) diag_point<R, D>(v, Vp, a, a.c0);
  if (a.rot_a) spin_mixing_point<R, D>(v, a.c1, a.tau_s, a.itp, st);
  if (a.nem_a) nematic_point<R, D>(v, a.c2, a.tau_s, a.itp);
  double bx = 0, by = 0, bz = 0;
  if (a.raman_a | a.raman_b) raman_field(a.rg, p, bx, by, bz);
  if (a.raman_a) spin_rotate<R, D>(v, (R)bx, (R)by, (R)bz, a.tau_r, a.itp, st);
  if (a.ddi_rot) {
    spin_rotate<R, D>(v, a.phi[p], a.phi[a.N + p], a.phi[2 * a.N + p], a.tau_ddi, a.itp, st);
  }
  if (a.raman_b) spin_rotate<R, D>(v, (R)bx, (R)by, (R)bz, a.tau_r, a.itp, st);
  if (a.nem_b) nematic_point<R, D>(v, a.c2, a.tau_s, a.itp);
  if (a.rot_b) spin_mixing_point<R, D>(v, a.c1, a.tau_s, a.itp, st);
  if (a.post_diag) diag_point<R, D>(v, Vp, a, a.c0);
#pragma unroll
  for (int c = 0; c < D; ++c) a.psi[c * a.N + p] = v[c];
  if (a.spin_out) {
    R fx, fy, fz;
    spin_vector<R, D>(v, st, fx, fy, fz);
    a.spin_out[p] = fx;
    a.spin_out[a.N + p] = fy;
    a.spin_out[2 * a.N + p] = fz;
  }
}

// ---------------------------------------------------------------------------
// Fused row pass for the no-DDI, no-tensor path: a tile of RPB x-rows (fixed y,z)
// with all D components in shared memory runs, in order and as selected by flags,
//   [scale by 1/sqrt(norm) (deferred ITP renormalisation)] [inverse x FFT]
//   [potential stage 1] [forward x FFT | 1-D kinetic step fwd*phase*inv]
//   [potential stage 2] [per-block sums of |psi|^2 for the next renormalisation]
// so a leapfrog step is this pass plus the last-axis pass (2-D) and psi makes one
// round trip through HBM/L2 per pass instead of one per operator.
// ---------------------------------------------------------------------------
enum RowFlags {
  RP_SCALE = 1,
  RP_INV_X = 2,
  RP_POT1 = 4,
  RP_FWD_X = 8,
  RP_KIN_X = 16,
  RP_POT2 = 32,
  RP_NORM = 64,
  RP_CORR = 128,  // multiply by corr[solve] on load (batched ITP: actual / predicted scale)
  RP_MID = 256    // after POT1: norm partial, multiply by pred[solve], POT2 (p2) — before FWD_X
};

// acc += |psi|^2 of one point (all D components), for the renormalisation sums of a row
// pass.  FP64: added to acc component by component in FP64.  FP32: the point's sum is formed
// in FP32 by FMAs (relative error a few units of 2^-24, without bias) and added once; the
// sums over points stay FP64.  Per element that is two FP32 FMAs instead of two conversions
// and three FP64 operations — on a part whose FP64 rate is 1/64 of FP32 the FP64 form made the
// closing ITP row pass FP64-bound.  The resulting scale is rounded to FP32 anyway (it
// multiplies FP32 data), which dominates the difference.
template <typename R, int D>
__device__ __forceinline__ void add_point_norm2(double& acc, const cplx<R> (&v)[D]) {
  if constexpr (sizeof(R) == 4) {
    float n = 0.0f;
#pragma unroll
    for (int c = 0; c < D; ++c) {
      n = fmaf(v[c].x, v[c].x, n);
      n = fmaf(v[c].y, v[c].y, n);
    }
    acc += (double)n;
  } else {
#pragma unroll
    for (int c = 0; c < D; ++c) acc += (double)v[c].x * v[c].x + (double)v[c].y * v[c].y;
  }
}

template <typename R>
struct RowArgs {
  cplx<R>* psi;
  int64_t N;          // points per component
  int64_t n_rows;     // N / nx
  int flags;
  PotArgs<R> p1, p2;  // potential stages (diag, spin mixing)
  const double* norm_total;  // per-solve sum |psi|^2 of the previous pass (RP_SCALE)
  double dV;
  double* partials;   // RP_NORM: one double per block
  // batches of independent solves (null active: a single solve)
  const int* active;        // slot -> solve index
  int blocks_per_solve;
  int64_t solve_stride;     // D*N elements between solves
  const R* c0s;             // per-solve couplings (null: p1/p2 values)
  const R* c1s;
  int n_slots;              // launch size: active slots (host side)
  const R* corr;            // RP_CORR
  const R* pred;            // RP_MID
};

template <typename R, int D>
__device__ __forceinline__ void pot_stage(cplx<R> (&v)[D], R Vp, const PotArgs<R>& a, const SpinTabs<R>& st, R c0,
                                          R c1) {
  const bool sm = a.rot_a && fabs(c1) >= (R)1e-30;
  if (a.pre_diag) diag_point<R, D>(v, Vp, a, c0);
  if (sm) spin_mixing_point<R, D>(v, c1, a.tau_s, a.itp, st);
  if (a.nem_a) nematic_point<R, D>(v, a.c2, a.tau_s, a.itp);
  if (a.nem_b) nematic_point<R, D>(v, a.c2, a.tau_s, a.itp);
  if (sm) spin_mixing_point<R, D>(v, c1, a.tau_s, a.itp, st);
  if (a.post_diag) diag_point<R, D>(v, Vp, a, c0);
}

// Threads of a row-pass block: enough for the FFTs (D*RPB lines of TPL threads) and
// for one point per thread in the potential stage, whichever is more.
template <typename R, int N, int D, int RPB, int P = 0>
constexpr int row_threads() {
  constexpr int fft = D * RPB * (N / PlanOf<R, N, P>::E);
  constexpr int pts = RPB * N;
  constexpr int t = fft > pts ? fft : (pts > 1024 ? 1024 : pts);
  return (t + 31) / 32 * 32;
}

// The work of row-pass block blk (CG and trig as in fft_strided_block).
template <typename R, int N, int D, int RPB, int P, bool PP, bool CG>
__device__ __forceinline__ void row_pass_block(const RowArgs<R>& a, const SpinTabs<R>& st, const PhaseRef<R>& ph,
                                               const Tw<R>& tw, int blk, unsigned char* smem_raw, bool trig) {
  constexpr int TPL = N / PlanOf<R, N, P>::E;
  constexpr int NL = D * RPB;  // line = c*RPB + r
  cplx<R>* s = reinterpret_cast<cplx<R>*>(smem_raw);
  cplx<R>* s2 = s + NL * N;  // second tile of the ping-pong stages (PP)
  __shared__ double red[32];
  const int tid = threadIdx.x;
  const int slot = a.active ? (int)(blk / a.blocks_per_solve) : 0;
  const int lblk = a.active ? (int)(blk % a.blocks_per_solve) : blk;
  const int b = a.active ? a.active[slot] : 0;
  cplx<R>* psi = a.psi + (int64_t)b * a.solve_stride;
  const R c0 = a.c0s ? a.c0s[b] : a.p1.c0;
  const R c1 = a.c1s ? a.c1s[b] : a.p1.c1;
  const int64_t row0 = (int64_t)lblk * RPB;
  const int nr = (int)min((int64_t)RPB, a.n_rows - row0);
  R scale = (R)1;
  if (a.flags & RP_SCALE) scale = (R)(1.0 / sqrt(a.norm_total[b] * a.dV));
  if (a.flags & RP_CORR) scale = a.corr[b];
  const bool scaled = (a.flags & (RP_SCALE | RP_CORR)) != 0;
  for (int f = tid; f < NL * N; f += blockDim.x) {
    const int line = f / N, x = f % N;
    const int c = line / RPB, r = line % RPB;
    cplx<R> v = mk<R>(0, 0);
    if (r < nr) v = ld_line<CG>(psi + c * a.N + (row0 + r) * N + x);
    if (scaled) v = v * scale;
    s[f] = v;
  }
  __syncthreads();
  const int t = tid % TPL, l = tid / TPL;
  const bool fa = l < NL;  // this thread works on an FFT line
  if (a.flags & RP_INV_X) fft_tile_sel<R, N, +1, P, PP>(s, s2, 1, N, l, t, tw, fa);
  double acc = 0.0;
  if (a.flags & RP_POT1) {
    const R pred = (a.flags & RP_MID) ? a.pred[b] : (R)1;
    for (int p = tid; p < RPB * N; p += blockDim.x) {
      const int r = p / N, x = p % N;
      if (r >= nr) continue;
      cplx<R> v[D];
#pragma unroll
      for (int c = 0; c < D; ++c) v[c] = s[(c * RPB + r) * N + x];
      const R Vp = a.p1.V[(row0 + r) * N + x];
      pot_stage<R, D>(v, Vp, a.p1, st, c0, c1);
      if (a.flags & RP_MID) {
        add_point_norm2<R, D>(acc, v);
#pragma unroll
        for (int c = 0; c < D; ++c) v[c] = v[c] * pred;
        pot_stage<R, D>(v, Vp, a.p2, st, c0, c1);
      }
#pragma unroll
      for (int c = 0; c < D; ++c) s[(c * RPB + r) * N + x] = v[c];
    }
    __syncthreads();
  }
  if (a.flags & (RP_FWD_X | RP_KIN_X)) fft_tile_sel<R, N, -1, P, PP>(s, s2, 1, N, l, t, tw, fa);
  if (a.flags & RP_KIN_X) {
    for (int f = tid; f < NL * N; f += blockDim.x) s[f] = phase_mul<R>(s[f], ph.tab[0], f % N, ph.scale0, ph.unbiased);
    __syncthreads();
    fft_tile_sel<R, N, +1, P, PP>(s, s2, 1, N, l, t, tw, fa);
  }
  if (a.flags & (RP_POT2 | RP_NORM)) {
    for (int p = tid; p < RPB * N; p += blockDim.x) {
      const int r = p / N, x = p % N;
      if (r >= nr) continue;
      cplx<R> v[D];
#pragma unroll
      for (int c = 0; c < D; ++c) v[c] = s[(c * RPB + r) * N + x];
      if (a.flags & RP_POT2) {
        pot_stage<R, D>(v, a.p2.V[(row0 + r) * N + x], a.p2, st, c0, c1);
#pragma unroll
        for (int c = 0; c < D; ++c) s[(c * RPB + r) * N + x] = v[c];
      }
      add_point_norm2<R, D>(acc, v);
    }
    __syncthreads();
  }
  if (trig) pdl_trigger();
  for (int f = tid; f < NL * N; f += blockDim.x) {
    const int line = f / N, x = f % N;
    const int c = line / RPB, r = line % RPB;
    if (r < nr) psi[c * a.N + (row0 + r) * N + x] = s[f];
  }
  if (a.flags & (RP_NORM | RP_MID)) {
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((tid & 31) == 0) red[tid >> 5] = acc;
    __syncthreads();
    if (tid == 0) {
      double x = 0.0;
      for (int w = 0; w < (int)((blockDim.x + 31) >> 5); ++w) x += red[w];
      a.partials[blk] = x;
    }
  }
}

template <typename R, int N, int D, int RPB, int P = 0, bool PP = false>
__global__ void __launch_bounds__(row_threads<R, N, D, RPB, P>())
k_row_pass(RowArgs<R> a, SpinTabs<R> st, PhaseRef<R> ph, Tw<R> tw) {
  pdl_wait();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  row_pass_block<R, N, D, RPB, P, PP, false>(a, st, ph, tw, (int)blockIdx.x, smem_raw, true);
}

// u[c][k] <- u[c][k+1], u[c][E-1] <- u[c][0]: after E calls u is back in its order.
template <typename R, int D, int E>
__device__ __forceinline__ void rotate_slots(cplx<R> (&u)[D][E]) {
#pragma unroll
  for (int c = 0; c < D; ++c) {
    const cplx<R> f = u[c][0];
#pragma unroll
    for (int k = 0; k + 1 < E; ++k) u[c][k] = u[c][k + 1];
    u[c][E - 1] = f;
  }
}

// Register-resident form of the fused row pass: the operators, flags and arithmetic of
// row_pass_block, with thread t of tile row rr holding positions x = t + k*TPL (k < E) of
// all D components of its row in registers.  Every x transform starts from and ends in
// registers (the first and last Stockham stages read and write exactly those positions,
// reg_fft_run), so psi is loaded from and stored to global memory directly (consecutive
// threads, consecutive x), the potential stages and the kinetic phase run on registers
// between the transforms, and shared memory carries only the transforms' inner stages
// (lines padded by one complex after every 16, RegRowIx): per pass half the shared-memory
// traffic and block barriers of the tile form, and no thread idles during a transform.
// The states are bit-identical to the tile form of the same plan; the norm partials
// (RP_NORM, RP_MID) are summed in another order.
template <typename R, int N, int D, int RPB, int P, bool PP>
__global__ void __launch_bounds__(RPB*(N / PlanOf<R, N, P>::E))
k_row_pass_reg(RowArgs<R> a, SpinTabs<R> st, PhaseRef<R> ph, Tw<R> tw) {
  constexpr int E = PlanOf<R, N, P>::E;
  constexpr int TPL = N / E;
  pdl_wait();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double red[32];
  cplx<R>* cur = reinterpret_cast<cplx<R>*>(smem_raw);
  cplx<R>* oth = cur + D * RPB * (N + N / 16);  // second tile of the ping-pong stages (PP)
  const RegRowIx ix{N + N / 16};
  const int tid = threadIdx.x;
  const int rr = tid / TPL, t = tid % TPL;
  const int blk = (int)blockIdx.x;
  const int slot = a.active ? (int)(blk / a.blocks_per_solve) : 0;
  const int lblk = a.active ? (int)(blk % a.blocks_per_solve) : blk;
  const int b = a.active ? a.active[slot] : 0;
  cplx<R>* psi = a.psi + (int64_t)b * a.solve_stride;
  const R c0 = a.c0s ? a.c0s[b] : a.p1.c0;
  const R c1 = a.c1s ? a.c1s[b] : a.p1.c1;
  const int64_t row = (int64_t)lblk * RPB + rr;
  const bool live = row < a.n_rows;
  R scale = (R)1;
  if (a.flags & RP_SCALE) scale = (R)(1.0 / sqrt(a.norm_total[b] * a.dV));
  if (a.flags & RP_CORR) scale = a.corr[b];
  const bool scaled = (a.flags & (RP_SCALE | RP_CORR)) != 0;
  cplx<R> u[D][E];
#pragma unroll
  for (int c = 0; c < D; ++c) {
#pragma unroll
    for (int k = 0; k < E; ++k) {
      cplx<R> v = mk<R>(0, 0);
      if (live) v = psi[c * a.N + row * N + t + k * TPL];
      if (scaled) v = v * scale;
      u[c][k] = v;
    }
  }
  // the potential at the thread's positions, loaded here so that the loads overlap the
  // inverse transform (rotated with u through the potential stage)
  R vp[E];
  const bool pot1 = (a.flags & RP_POT1) != 0;
#pragma unroll
  for (int k = 0; k < E; ++k) vp[k] = (pot1 && live) ? a.p1.V[row * N + t + k * TPL] : (R)0;
  const int l0 = rr * D;
  if (a.flags & RP_INV_X) PlanOf<R, N, P>::template run_reg<R, +1, PP, D>(u, cur, oth, ix, l0, t, tw);
  // The pointwise stages take the thread's E points one after another through slot 0 of u
  // (rotate_slots): a runtime loop keeps one copy of the stage's code, where unrolling
  // over the points would inline the potential stage E times per flag.
  double acc = 0.0;
  if (a.flags & RP_POT1) {
    const R pred = (a.flags & RP_MID) ? a.pred[b] : (R)1;
#pragma unroll 1
    for (int k = 0; k < E; ++k) {
      if (live) {
        cplx<R> v[D];
#pragma unroll
        for (int c = 0; c < D; ++c) v[c] = u[c][0];
        const R Vp = vp[0];
        pot_stage<R, D>(v, Vp, a.p1, st, c0, c1);
        if (a.flags & RP_MID) {
          add_point_norm2<R, D>(acc, v);
#pragma unroll
          for (int c = 0; c < D; ++c) v[c] = v[c] * pred;
          pot_stage<R, D>(v, Vp, a.p2, st, c0, c1);
        }
#pragma unroll
        for (int c = 0; c < D; ++c) u[c][0] = v[c];
      }
      rotate_slots<R, D, E>(u);
      {
        const R f = vp[0];
#pragma unroll
        for (int q = 0; q + 1 < E; ++q) vp[q] = vp[q + 1];
        vp[E - 1] = f;
      }
    }
  }
  if (a.flags & (RP_FWD_X | RP_KIN_X)) PlanOf<R, N, P>::template run_reg<R, -1, PP, D>(u, cur, oth, ix, l0, t, tw);
  if (a.flags & RP_KIN_X) {
#pragma unroll
    for (int c = 0; c < D; ++c) {
#pragma unroll
      for (int k = 0; k < E; ++k) u[c][k] = phase_mul<R>(u[c][k], ph.tab[0], t + k * TPL, ph.scale0, ph.unbiased);
    }
    PlanOf<R, N, P>::template run_reg<R, +1, PP, D>(u, cur, oth, ix, l0, t, tw);
  }
  if (a.flags & (RP_POT2 | RP_NORM)) {
#pragma unroll 1
    for (int k = 0; k < E; ++k) {
      if (live) {
        if (a.flags & RP_POT2) {
          cplx<R> v[D];
#pragma unroll
          for (int c = 0; c < D; ++c) v[c] = u[c][0];
          pot_stage<R, D>(v, a.p2.V[row * N + t + k * TPL], a.p2, st, c0, c1);
#pragma unroll
          for (int c = 0; c < D; ++c) u[c][0] = v[c];
        }
        {
          cplx<R> v[D];
#pragma unroll
          for (int c = 0; c < D; ++c) v[c] = u[c][0];
          add_point_norm2<R, D>(acc, v);
        }
      }
      rotate_slots<R, D, E>(u);
    }
  }
  pdl_trigger();
  if (live) {
#pragma unroll
    for (int c = 0; c < D; ++c) {
#pragma unroll
      for (int k = 0; k < E; ++k) psi[c * a.N + row * N + t + k * TPL] = u[c][k];
    }
  }
  if (a.flags & (RP_NORM | RP_MID)) {
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((tid & 31) == 0) red[tid >> 5] = acc;
    __syncthreads();
    if (tid == 0) {
      double x = 0.0;
      for (int w = 0; w < (int)((blockDim.x + 31) >> 5); ++w) x += red[w];
      a.partials[blk] = x;
    }
  }
}

// n fused ITP split steps of a 1-D solve (one row-pass block holds its whole line of all
// components) in one launch: each iteration is the row pass of fused_steps_body (V/2, kinetic,
// V/2, norm partial), the block's partial is the solve's norm (what the one-block finish of
// the separate launches writes), and the next iteration scales by it.  The state is
// bit-identical to the launch-per-step sequence; the last step's renormalisation is left
// pending in norm_out, as there.
template <typename R, int N, int D, int RPB, int P = 0, bool PP = false>
__global__ void __launch_bounds__(row_threads<R, N, D, RPB, P>())
k_row_itp_steps(RowArgs<R> a, SpinTabs<R> st, PhaseRef<R> ph, Tw<R> tw, long long n_steps, int first_pending,
                double* norm_out) {
  pdl_wait();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int base = a.flags;
  for (long long step = 0; step < n_steps; ++step) {
    a.flags = base | ((step > 0 || first_pending) ? RP_SCALE : 0);
    row_pass_block<R, N, D, RPB, P, PP, false>(a, st, ph, tw, 0, smem_raw, false);
    __syncthreads();  // psi stores and the partial are visible to the whole block
    if (threadIdx.x == 0) norm_out[0] = a.partials[0];
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Persistent leapfrog segment (src/simulation.jl:49-94, the merged steps between save
// points) for 2-D grids: one cooperative launch runs n steps, each the kinetic column
// pass (y FFT, kinetic phase, inverse y FFT) and the row pass (inverse x FFT, full
// potential step, forward x FFT), separated by grid-wide barriers instead of kernel
// boundaries.  Every block does the same per-line work as the separate kernels with
// the same plan, so the state is bit-identical to theirs.
// ---------------------------------------------------------------------------
struct GridBarrier {
  unsigned int count;  // blocks arrived at the current barrier
  unsigned int gen;    // barriers completed
  int err;             // 1: a wait ran out (the launch then returns early)
  int pad;
};

constexpr unsigned int kBarrierSpinLimit = 1u << 20;  // 0.1-1 s of polling (100 ns sleeps)

// Grid-wide barrier of a cooperative launch (all blocks resident).  Thread 0 of each
// block arrives with a release fence and waits, polling with a bounded count, for the
// last arriver to advance the generation; on a timeout (or another block's) it records
// the error and the block returns false.
__device__ __forceinline__ bool grid_barrier(GridBarrier* b) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned int* gen = &b->gen;
    volatile int* err = &b->err;
    int good = *err == 0;
    if (good) {
      const unsigned int g = *gen;
      __threadfence();
      if (atomicAdd(&b->count, 1u) == gridDim.x - 1) {
        atomicExch(&b->count, 0u);
        __threadfence();
        atomicAdd(&b->gen, 1u);
      } else {
        unsigned int spins = 0;
        while (*gen == g) {
          if (*err != 0) {
            good = 0;
            break;
          }
          if (++spins > kBarrierSpinLimit) {
            atomicExch(&b->err, 1);
            good = 0;
            break;
          }
          __nanosleep(100);
        }
      }
      __threadfence();
    }
    ok = good;
  }
  __syncthreads();
  return ok != 0;
}

// Tile shapes of the segment kernel: the row pass of the default plan, and as many
// y columns per block as fill the same thread count.
template <typename R, int NX, int NY, int D, int P>
struct SegShape {
  static constexpr int TPLX = NX / PlanOf<R, NX, P>::E;
  static constexpr int TPLY = NY / PlanOf<R, NY, P>::E;
  static constexpr int RPB = (64 / (D * TPLX)) < 1 ? 1 : 64 / (D * TPLX);
  static constexpr int T = row_threads<R, NX, D, RPB, P>();
  static constexpr int W = T / TPLY;
  static_assert(W * TPLY == T, "segment tiles need T divisible by the y line's threads");
  static constexpr int TILE = (D * RPB * NX > W * NY) ? D * RPB * NX : W * NY;
  static constexpr size_t smem_bytes = 2 * (size_t)TILE * sizeof(cplx<R>);  // ping-pong stages
};

template <typename R, int NX, int NY, int D, int P>
__global__ void __launch_bounds__(SegShape<R, NX, NY, D, P>::T)
k_lf_segment(RowArgs<R> a, SpinTabs<R> st, PhaseRef<R> ph, Tw<R> twx, Tw<R> twy, long long n_steps,
             GridBarrier* bar) {
  using Sh = SegShape<R, NX, NY, D, P>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int row_units = (int)((a.n_rows + Sh::RPB - 1) / Sh::RPB);
  constexpr int col_per = (NX + Sh::W - 1) / Sh::W;  // column tiles per component
  const int col_units = col_per * D;
  for (long long step = 0; step < n_steps; ++step) {
    for (int u = blockIdx.x; u < col_units; u += gridDim.x) {
      fft_strided_block<R, NY, Sh::W, P, true, true>(a.psi, NX, NX, a.N, NY, NY, 2, ph, twy,
                                                     (int64_t)(u % col_per) * Sh::W, u / col_per, smem_raw, false);
      __syncthreads();
    }
    if (!grid_barrier(bar)) return;
    for (int u = blockIdx.x; u < row_units; u += gridDim.x) {
      row_pass_block<R, NX, D, Sh::RPB, P, true, true>(a, st, ph, twx, u, smem_raw, false);
      __syncthreads();
    }
    if (step + 1 < n_steps && !grid_barrier(bar)) return;
  }
}

// ---------------------------------------------------------------------------
// General-F tensor interaction (src/tensor_interaction.jl:130-240).
// h_{cc'} = sum_J G[J][c][c'] conj(psi_{J-c}) psi_{J-c'} with
// G[J][c][c'] = sum_S g_S CG(m,mu|S,M) CG(m',nu|S,M), M = 2F - J (the HF-entry sum
// regrouped by M; same terms, fewer multiplies).  psi <- exp(-i h tau) psi is
// evaluated by a Taylor series with sub-steps sized from the bound
// ||h|| <= n * sum_S |g_S| (2S+1)/(2F+1); the series is cut when the bound of the
// next term falls below the working precision.  exp(-i h tau) is the same
// operator the reference forms from the eigen-decomposition V e^{-i Lambda tau} V^†.
// ---------------------------------------------------------------------------
template <typename R>
struct TensorArgs {
  cplx<R>* psi;
  int64_t N;
  const R* V;
  const double* G;            // (4F+1) * D * D
  const float* G32;           // the same coefficients in FP32 (FP32 form; null in FP64)
  double bound_coef;          // sum_S |g_S| (2S+1)/(2F+1)
  int n_apply;                // 1 or 2 tensor applications
  int pre_diag, post_diag;
  int itp;
  R tau;                      // tensor tau
  R tau_d, c0, c_lhy;         // diagonal stage (same layout as PotArgs)
  cplx<R> zee[kMaxD];
  cplx<R> zee_lo[kMaxD];
  double eps;                 // series cut
};

template <typename R, int D>
__device__ __forceinline__ void diag_point_t(cplx<R> (&v)[D], R Vp, const TensorArgs<R>& a) {
  R n = 0;
#pragma unroll
  for (int c = 0; c < D; ++c) n += abs2(v[c]);
  R Vint = a.c0 * n;
  if (a.c_lhy != (R)0) Vint += a.c_lhy * n * sqrt(n);
  diag_apply<R, D>(v, Vp + Vint, a.tau_d, a.itp, a.zee, a.zee_lo);
}

template <typename R, int D>
__device__ __forceinline__ void tensor_point(cplx<R> (&v)[D], const TensorArgs<R>& a, cplx<R>* hs, int hstride) {
  constexpr int F = (D - 1) / 2;
  R nl = 0;
#pragma unroll
  for (int c = 0; c < D; ++c) nl += abs2(v[c]);
  if (nl < (R)1e-20) return;
  // build the upper triangle of h into shared memory
  int hi = 0;
#pragma unroll
  for (int c = 0; c < D; ++c) {
#pragma unroll
    for (int cp = c; cp < D; ++cp) {
      cplx<R> acc = mk<R>(0, 0);
#pragma unroll
      for (int J = cp; J <= c + D - 1; ++J) {
        const R gcoef = (R)__ldg(a.G + ((size_t)J * D + c) * D + cp);
        acc += gcoef * cmulc(v[J - c], v[J - cp]);
      }
      if (c == cp) acc.y = (R)0;  // h is Hermitian: a real diagonal (not the rounding residual of conj(v) v)
      hs[hi * hstride] = acc;
      ++hi;
    }
  }
  const double x = a.bound_coef * (double)nl * fabs((double)a.tau);
  int nsub = 1;
  if (x > 0.5) nsub = x < 0.5 * kMaxSub ? (int)ceil(x / 0.5) : kMaxSub;  // bounded for non-finite states
  const double xs = x / nsub;
  // number of terms: smallest K with xs^(K+1)/(K+1)! < eps
  int K = 0;
  {
    double term = 1.0;
    while (K < 40) {
      term *= xs / (double)(K + 1);
      if (term < a.eps) break;
      ++K;
    }
    K = K + 1;
  }
  // Horner's scheme (as in rotate_taylor): y <- v + (-i dtau / k) h y for k = K..1.
  const R dtau = a.tau / (R)nsub;
  for (int sub = 0; sub < nsub; ++sub) {
    cplx<R> y[D];
#pragma unroll
    for (int c = 0; c < D; ++c) y[c] = v[c];
    for (int k = K; k >= 1; --k) {
      cplx<R> t[D];
#pragma unroll
      for (int c = 0; c < D; ++c) t[c] = mk<R>(0, 0);
      int idx = 0;
#pragma unroll
      for (int c = 0; c < D; ++c) {
#pragma unroll
        for (int cp = c; cp < D; ++cp) {
          const cplx<R> h = hs[idx * hstride];
          t[c] += h * y[cp];
          if (cp != c) t[cp] += cmulc(h, y[c]);
          ++idx;
        }
      }
      const R f = dtau / (R)k;
#pragma unroll
      for (int c = 0; c < D; ++c) y[c] = v[c] + (a.itp ? (-f) * t[c] : mul_mi(f * t[c]));
    }
#pragma unroll
    for (int c = 0; c < D; ++c) v[c] = y[c];
  }
  (void)F;
}

template <typename R, int D>
__global__ void __launch_bounds__(64) k_tensor(TensorArgs<R> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<R>* hs = reinterpret_cast<cplx<R>*>(smem_raw) + threadIdx.x;
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.N) return;
  cplx<R> v[D];
#pragma unroll
  for (int c = 0; c < D; ++c) v[c] = a.psi[c * a.N + p];
  const R Vp = a.V[p];
  if (a.pre_diag) diag_point_t<R, D>(v, Vp, a);
  for (int r = 0; r < a.n_apply; ++r) tensor_point<R, D>(v, a, hs, blockDim.x);
  if (a.post_diag) diag_point_t<R, D>(v, Vp, a);
#pragma unroll
  for (int c = 0; c < D; ++c) a.psi[c * a.N + p] = v[c];
}

// ---------------------------------------------------------------------------
// FP32 tensor step with one group of L lanes per point (lane c holds components c, c + L,
// ... — RL of them): the same operator as tensor_point, laid out for occupancy.  One thread
// per point needs the whole 13-component spinor, h and the series terms in registers (255
// and spills for F = 6) and keeps 8 warps per SM resident; here each lane holds RL rows of
// h, the upper triangle of h is built cooperatively (entries round-robin over the lanes,
// lower entries taken as conjugates so h stays exactly Hermitian) and each Horner product
// broadcasts the vector through a double-buffered shared slot (D loads per lane and step
// for RL rows of D complex products: RL = 2 doubles the arithmetic per shared load).
// After the block-wide staging of G, groups synchronise only among their own lanes.
// ---------------------------------------------------------------------------
template <int D, int RL = 1>
struct TensorLanes {
  // lanes per point: one row of h per lane (8 or 16 lanes), or RL rows per lane (the power of
  // two at or above ceil(D / RL)); lane c owns components c, c + L, ...
  static constexpr int L = RL == 1 ? (D <= 8 ? 8 : 16)
                                   : ((D + RL - 1) / RL <= 2 ? 2 : (D + RL - 1) / RL <= 4 ? 4 : (D + RL - 1) / RL <= 8 ? 8 : 16);
  static constexpr int YB = L * RL;          // entries of one vector buffer (>= D)
  // per-group stride of the two vector buffers: one entry of padding, so that the groups of
  // a warp reading their own y_j in the same Horner step hit different banks (at 2 YB, a
  // multiple of 32 words, they all hit one)
  static constexpr int YS = 2 * YB + 1;
  static constexpr int PPB = 256 / L;        // points per 256-thread block
  static constexpr int NJ = 2 * D - 1;
  static constexpr int NT = D * (D + 1) / 2;  // upper-triangle entries
  static constexpr int G_FLOATS = (NJ * D * D + 3) / 4 * 4;
  static constexpr int E_INTS = (NT + 3) / 4 * 4;
  static constexpr size_t smem_bytes() {
    return sizeof(float) * G_FLOATS + sizeof(int) * E_INTS + sizeof(float2) * (size_t)PPB * (NT + D * D + YS);
  }
};

template <int L>
__device__ __forceinline__ float group_sum(float x, unsigned mask) {
#pragma unroll
  for (int o = L / 2; o > 0; o >>= 1) x += __shfl_xor_sync(mask, x, o);
  return x;
}

template <int D, int L, int RL>
__device__ __forceinline__ void diag_lane(float2 (&v)[RL], float Vp, const TensorArgs<float>& a, int c,
                                          unsigned mask) {
  float s = 0.0f;
#pragma unroll
  for (int r = 0; r < RL; ++r)
    if (c + L * r < D) s += abs2(v[r]);
  const float n = group_sum<L>(s, mask);
  float Vint = a.c0 * n;
  if (a.c_lhy != 0.0f) Vint += a.c_lhy * n * sqrtf(n);
  const float veff = Vp + Vint;
#pragma unroll
  for (int r = 0; r < RL; ++r) {
    const int comp = c + L * r;
    if (comp >= D) continue;
    if (a.itp) {
      v[r] = v[r] * (expf(-veff * a.tau_d) * a.zee[comp].x);
    } else {
      float sn, cm1;
      sin_cosm1(veff * a.tau_d, sn, cm1);
      v[r] = rot_small_zee(v[r], cm1, sn, a.zee_lo[comp]);
    }
  }
}

template <int D, int L, int RL>
__device__ __forceinline__ void tensor_lane(float2 (&v)[RL], const TensorArgs<float>& a, const float* Gs,
                                            const int* Ent, float2* Ps, float2* Hs, float2* Ys, int c, unsigned mask) {
  constexpr int NT = D * (D + 1) / 2;
  constexpr int YB = L * RL;
  float s = 0.0f;
#pragma unroll
  for (int r = 0; r < RL; ++r)
    if (c + L * r < D) s += abs2(v[r]);
  const float nl = group_sum<L>(s, mask);
  if (nl < 1e-20f) return;
#pragma unroll
  for (int r = 0; r < RL; ++r)
    if (c + L * r < D) Ys[c + L * r] = v[r];
  __syncwarp(mask);
  // products P[b][a] = conj(v_b) v_a (b <= a), upper-triangle storage, row b from b*D - b(b-1)/2;
  // P[b][b] = |v_b|^2 exactly real (the fused form of conj(v) v keeps the rounding residual of
  // x y as an imaginary part, which would make the diagonal of h complex and the step
  // non-unitary)
  for (int e = c; e < NT; e += L) {
    const int b = Ent[e] & 0xff, aa = Ent[e] >> 8;
    Ps[b * D - b * (b - 1) / 2 + (aa - b)] = b == aa ? mk<float>(abs2(Ys[b]), 0.0f) : cmulc(Ys[b], Ys[aa]);
  }
  __syncwarp(mask);
  // h[i][j] (j >= i) = sum_{J=j}^{i+D-1} G[J][i][j] conj(v[J-i]) v[J-j] = sum G conj(P[J-j][J-i]);
  // entries ordered by diagonal (equal term counts in each round of the lanes)
  for (int e = c; e < NT; e += L) {
    const int i = Ent[e] & 0xff, j = Ent[e] >> 8;
    float2 acc = mk<float>(0.0f, 0.0f);
    int bq = 0;                                   // b = J - j, a = J - i = b + (j - i)
    int idx = (j - i);                            // index of P[0][j-i]
    const float* g = Gs + (j * D + i) * D + j;    // G[J][i][j] at J = j
    for (int J = j; J <= i + D - 1; ++J) {
      const float2 p = Ps[idx];
      const float gv = *g;
      acc.x = fmaf(gv, p.x, acc.x);
      acc.y = fmaf(-gv, p.y, acc.y);
      idx += D - bq;
      ++bq;
      g += D * D;
    }
    Hs[i * D + j] = acc;
  }
  __syncwarp(mask);
  float2 hrow[RL][D];
#pragma unroll
  for (int r = 0; r < RL; ++r) {
    const int comp = c + L * r;
#pragma unroll
    for (int j = 0; j < D; ++j)
      hrow[r][j] = comp >= D ? mk<float>(0.0f, 0.0f) : (j >= comp ? Hs[comp * D + j] : conj(Hs[j * D + comp]));
  }
  const double x = a.bound_coef * (double)nl * fabs((double)a.tau);
  int nsub = 1;
  if (x > 0.5) nsub = x < 0.5 * kMaxSub ? (int)ceil(x / 0.5) : kMaxSub;  // bounded for non-finite states
  const double xs = x / nsub;
  int K = 0;
  {
    double term = 1.0;
    while (K < 40) {
      term *= xs / (double)(K + 1);
      if (term < a.eps) break;
      ++K;
    }
    K = K + 1;
  }
  const float dtau = a.tau / (float)nsub;
  for (int sub = 0; sub < nsub; ++sub) {
    float2 y[RL];
#pragma unroll
    for (int r = 0; r < RL; ++r) y[r] = v[r];
    for (int k = K; k >= 1; --k) {
      float2* yb = Ys + (k & 1) * YB;
#pragma unroll
      for (int r = 0; r < RL; ++r)
        if (c + L * r < D) yb[c + L * r] = y[r];
      __syncwarp(mask);
      const float f = dtau / (float)k;
#pragma unroll
      for (int r = 0; r < RL; ++r) {
        const int comp = c + L * r;
        float2 t = mk<float>(0.0f, 0.0f);
#pragma unroll
        for (int j = 0; j < D; ++j) t += hrow[r][j] * yb[j];
        if (k == 1 && !a.itp) {
          // unbiased rounding of the last addition (as in rotate_taylor)
          const float2 corr = mul_mi(f * t);
          y[r] = mk<float>(sr_add(v[r].x, corr.x, 0x27d4eb2fu + 0x165667b1u * comp),
                           sr_add(v[r].y, corr.y, 0x9e3779b1u + 0x85ebca77u * comp));
        } else {
          y[r] = v[r] + (a.itp ? (-f) * t : mul_mi(f * t));
        }
      }
    }
#pragma unroll
    for (int r = 0; r < RL; ++r) v[r] = y[r];
  }
  __syncwarp(mask);
}

// ---------------------------------------------------------------------------
// FP32 tensor step with rows of h in registers (k_tensor_rows): a block of NW warps serves
// 32 points, one point per lane (launched with NW = (D + 1) / 2: two rows per warp); warp q
// builds and keeps rows i = q, q + NW, ... of its points' h in registers, and every warp holds
// the whole spinor, so all register indices are compile-time (the warp's rows are template
// arguments, chosen by a warp-uniform dispatch) and the G coefficients are read at
// warp-uniform addresses (broadcast).  A Horner step multiplies the warp's rows by the vector
// and exchanges the new entries through shared memory (double-buffered, one block barrier per
// step).  h_ij for i > j is formed from the same coefficient G[J][j][i] and the same rounded
// products as h_ji, so h is exactly Hermitian.  Sub-step count and series length are the
// block's maxima (uniform trip counts around the barriers; extra terms only shorten the
// truncation).
// ---------------------------------------------------------------------------
template <int D, int NW, int Q>
__device__ __forceinline__ void tensor_rows_apply(float2 (&v)[D], const TensorArgs<float>& a, float2* ys, int lane,
                                                  bool act, int nsub, int K, float dtau) {
  constexpr int R = (D - Q + NW - 1) / NW;  // rows Q, Q + NW, ... < D
  float2 h[R > 0 ? R : 1][D];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int i = Q + NW * r;
#pragma unroll
    for (int j = 0; j < D; ++j) {
      const int lo = i < j ? i : j, hi = i < j ? j : i;
      float ax = 0.0f, ay = 0.0f;
#pragma unroll
      for (int J = hi; J <= lo + D - 1; ++J) {
        const float g = __ldg(a.G32 + ((size_t)J * D + lo) * D + hi);
        const float2 u = v[J - i], w = v[J - j];
        // conj(u) w with separately rounded products: the (j, i) entry uses the same
        // products, so it is the exact conjugate
        const float pr = __fadd_rn(__fmul_rn(u.x, w.x), __fmul_rn(u.y, w.y));
        const float pi = __fsub_rn(__fmul_rn(u.x, w.y), __fmul_rn(u.y, w.x));
        ax = fmaf(g, pr, ax);
        ay = fmaf(g, pi, ay);
      }
      h[r][j] = make_float2(ax, ay);
    }
  }
  for (int sub = 0; sub < nsub; ++sub) {
    float2 y[D];
#pragma unroll
    for (int c = 0; c < D; ++c) y[c] = v[c];
    for (int k = K; k >= 1; --k) {
      float2* yb = ys + (k & 1) * D * 32;
      const float f = dtau / (float)k;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int i = Q + NW * r;
        float2 t = make_float2(0.0f, 0.0f);
#pragma unroll
        for (int j = 0; j < D; ++j) t += h[r][j] * y[j];
        float2 yn;
        if (a.itp) {
          yn = v[i] + (-f) * t;
        } else if (k == 1) {
          const float2 corr = mul_mi(f * t);  // unbiased last addition, as in rotate_taylor
          yn = make_float2(sr_add(v[i].x, corr.x, 0x27d4eb2fu + 0x165667b1u * i),
                           sr_add(v[i].y, corr.y, 0x9e3779b1u + 0x85ebca77u * i));
        } else {
          yn = v[i] + mul_mi(f * t);
        }
        yb[i * 32 + lane] = yn;
      }
      __syncthreads();
#pragma unroll
      for (int c = 0; c < D; ++c) y[c] = yb[c * 32 + lane];
    }
#pragma unroll
    for (int c = 0; c < D; ++c)
      if (act) v[c] = y[c];
    __syncthreads();  // every warp has read this sub-step's last exchange before the next one writes
  }
}

// Runs warp q's instance (a warp-uniform branch: one template instance per warp).
template <int D, int NW, int Q>
__device__ __forceinline__ void tensor_rows_dispatch(int q, float2 (&v)[D], const TensorArgs<float>& a, float2* ys,
                                                     int lane, bool act, int nsub, int K, float dtau) {
  if constexpr (Q < NW) {
    if (q == Q) {
      tensor_rows_apply<D, NW, Q>(v, a, ys, lane, act, nsub, K, dtau);
      return;
    }
    tensor_rows_dispatch<D, NW, Q + 1>(q, v, a, ys, lane, act, nsub, K, dtau);
  }
}

template <int D, int NW>
__global__ void __launch_bounds__(32 * NW) k_tensor_rows(TensorArgs<float> a) {
  __shared__ float2 ys[2 * D * 32];
  const int lane = threadIdx.x & 31, q = threadIdx.x >> 5;
  const int64_t p = (int64_t)blockIdx.x * 32 + lane;
  const bool inb = p < a.N;
  float2 v[D];
#pragma unroll
  for (int c = 0; c < D; ++c) v[c] = inb ? a.psi[c * a.N + p] : make_float2(0.0f, 0.0f);
  const float Vp = inb ? a.V[p] : 0.0f;
  if (a.pre_diag) diag_point_t<float, D>(v, Vp, a);
  for (int rep = 0; rep < a.n_apply; ++rep) {
    float nl = 0.0f;
#pragma unroll
    for (int c = 0; c < D; ++c) nl += abs2(v[c]);
    const bool act = inb && nl >= 1e-20f;
    // sub-steps and series length: the block's maxima (every warp holds the same 32 points)
    double x = act ? a.bound_coef * (double)nl * fabs((double)a.tau) : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x = fmax(x, __shfl_xor_sync(0xffffffffu, x, o));
    int nsub = 1;
    if (x > 0.5) nsub = x < 0.5 * kMaxSub ? (int)ceil(x / 0.5) : kMaxSub;  // bounded for non-finite states
    const double xs = x / nsub;
    int K = 0;
    {
      double term = 1.0;
      while (K < 40) {
        term *= xs / (double)(K + 1);
        if (term < a.eps) break;
        ++K;
      }
      K = K + 1;
    }
    const float dtau = a.tau / (float)nsub;
    tensor_rows_dispatch<D, NW, 0>(q, v, a, ys, lane, act, nsub, K, dtau);
  }
  if (a.post_diag) diag_point_t<float, D>(v, Vp, a);
  if (!inb) return;
#pragma unroll
  for (int c = 0; c < D; ++c)
    if (c % NW == q) a.psi[c * a.N + p] = v[c];
}

template <int D, int RL>
__global__ void __launch_bounds__(256) k_tensor_lanes(TensorArgs<float> a) {
  using TL = TensorLanes<D, RL>;
  constexpr int L = TL::L;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* Gs = reinterpret_cast<float*>(smem_raw);
  int* Ent = reinterpret_cast<int*>(Gs + TL::G_FLOATS);
  float2* Psb = reinterpret_cast<float2*>(Ent + TL::E_INTS);
  float2* Hs = Psb + TL::PPB * TL::NT;
  float2* Ysb = Hs + TL::PPB * D * D;
  const int tid = threadIdx.x;
  for (int i = tid; i < TL::NJ * D * D; i += blockDim.x) Gs[i] = (float)a.G[i];
  if (tid < TL::NT) {
    // entry tid in diagonal order: d = j - i, then i; packed as i | (j << 8)
    int e = tid, d = 0;
    while (e >= D - d) {
      e -= D - d;
      ++d;
    }
    Ent[tid] = e | ((e + d) << 8);
  }
  __syncthreads();
  const int g = tid / L, c = tid % L;
  const int64_t p = (int64_t)blockIdx.x * TL::PPB + g;
  if (p >= a.N) return;  // the whole group leaves; only group-local synchronisation follows
  const unsigned mask = ((L == 32) ? 0xffffffffu : ((1u << L) - 1u)) << ((tid & 31) / L * L);
  float2 v[RL];
#pragma unroll
  for (int r = 0; r < RL; ++r) v[r] = c + L * r < D ? a.psi[(c + L * r) * a.N + p] : mk<float>(0.0f, 0.0f);
  const float Vp = a.V[p];
  if (a.pre_diag) diag_lane<D, L, RL>(v, Vp, a, c, mask);
  for (int r = 0; r < a.n_apply; ++r)
    tensor_lane<D, L, RL>(v, a, Gs, Ent, Psb + g * TL::NT, Hs + g * D * D, Ysb + g * TL::YS, c, mask);
  if (a.post_diag) diag_lane<D, L, RL>(v, Vp, a, c, mask);
#pragma unroll
  for (int r = 0; r < RL; ++r)
    if (c + L * r < D) a.psi[(c + L * r) * a.N + p] = v[r];
}

// Spin density only (src/observables.jl:61-86).
template <typename R, int D>
__global__ void __launch_bounds__(256) k_spin_density(const cplx<R>* __restrict__ psi, int64_t N, SpinTabs<R> st,
                                                      R* __restrict__ out) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= N) return;
  cplx<R> v[D];
#pragma unroll
  for (int c = 0; c < D; ++c) v[c] = psi[c * N + p];
  R fx, fy, fz;
  spin_vector<R, D>(v, st, fx, fy, fz);
  out[p] = fx;
  out[N + p] = fy;
  out[2 * N + p] = fz;
}

// Density-dependent loss (src/losses.jl:25-45): psi_c *= exp(-rate_c n dt/2) with n the total
// density before the step; components with rate_c < 1e-30 are left as they are.
template <typename R>
struct LossRates {
  R r[kMaxD];
};
template <typename R, int D>
__global__ void __launch_bounds__(256) k_loss(cplx<R>* __restrict__ psi, int64_t N, LossRates<R> rates, R half_dt) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= N) return;
  cplx<R> v[D];
  R n = 0;
#pragma unroll
  for (int c = 0; c < D; ++c) {
    v[c] = psi[c * N + p];
    n += v[c].x * v[c].x + v[c].y * v[c].y;
  }
#pragma unroll
  for (int c = 0; c < D; ++c) {
    if (!(rates.r[c] >= (R)1e-30)) continue;
    const R f = exp(-rates.r[c] * n * half_dt);
    psi[c * N + p] = mk<R>(v[c].x * f, v[c].y * f);
  }
}

// f+(m_c) = sqrt(F(F+1) - m_c(m_c+1)) in FP64 for the FP64 reductions: the SpinTabs copy
// is rounded to the working precision, which in the FP32 form would put a 1e-8 relative
// error into every <Fx>, <Fy> sum.
template <int D>
__device__ __forceinline__ double fp_exact(int c) {
  constexpr int F = (D - 1) / 2;
  const int m = F - c;
  return sqrt((double)(F * (F + 1) - m * (m + 1)));
}

// ---------------------------------------------------------------------------
// Reductions: per-block partial results (double), then a fixed-order finish.
// ---------------------------------------------------------------------------
constexpr int kRedThreads = 256;

template <int K>
__device__ __forceinline__ void block_reduce_store(double (&vals)[K], double* partials, bool is_max) {
  __shared__ double red[K][kRedThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    double x = vals[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double y = __shfl_down_sync(0xffffffffu, x, o);
      x = is_max ? fmax(x, y) : x + y;
    }
    if (lane == 0) red[k][warp] = x;
  }
  __syncthreads();
  if (threadIdx.x < K) {
    const int k = threadIdx.x;
    double x = red[k][0];
    for (int w = 1; w < kRedThreads / 32; ++w) x = is_max ? fmax(x, red[k][w]) : x + red[k][w];
    partials[(size_t)blockIdx.x * K + k] = x;
  }
}

// Sum (or max) K values over nb partial blocks into out[k].
template <int K>
__global__ void k_reduce_finish(const double* __restrict__ partials, int nb, int is_max, double* __restrict__ out) {
  pdl_wait();
  const int k = threadIdx.x;
  if (k >= K) return;
  double x = is_max ? 0.0 : 0.0;
  for (int b = 0; b < nb; ++b) {
    const double y = partials[(size_t)b * K + k];
    x = is_max ? fmax(x, y) : x + y;
  }
  out[k] = x;
}

// Per-component sums of |psi_c|^2 (D values) and the NaN count (slot D).
template <typename R, int D>
__global__ void __launch_bounds__(kRedThreads) k_comp_norms(const cplx<R>* __restrict__ psi, int64_t N,
                                                            double* partials) {
  double acc[D + 1];
#pragma unroll
  for (int c = 0; c <= D; ++c) acc[c] = 0.0;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < N; p += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
    for (int c = 0; c < D; ++c) {
      const cplx<R> z = psi[c * N + p];
      acc[c] += (double)z.x * (double)z.x + (double)z.y * (double)z.y;
      if (isnan(z.x) || isnan(z.y)) acc[D] += 1.0;
    }
  }
  block_reduce_store<D + 1>(acc, partials, false);
}

// Energy terms on the grid: [trap, n^2, |f|^2, n^{5/2}] (src/energy.jl:67-108).
template <typename R, int D>
__global__ void __launch_bounds__(kRedThreads) k_energy_local(const cplx<R>* __restrict__ psi, int64_t N,
                                                              const R* __restrict__ V, SpinTabs<R> st,
                                                              double* partials) {
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < N; p += (int64_t)gridDim.x * blockDim.x) {
    double n = 0.0, fz = 0.0, fre = 0.0, fim = 0.0;
    cplx<R> prev = mk<R>(0, 0);
#pragma unroll
    for (int c = 0; c < D; ++c) {
      const cplx<R> z = psi[c * N + p];
      const double a2 = (double)z.x * z.x + (double)z.y * z.y;
      n += a2;
      fz += (double)st.m[c] * a2;
      if (c >= 1) {
        const double pr = (double)prev.x * z.x + (double)prev.y * z.y;
        const double pi = (double)prev.x * z.y - (double)prev.y * z.x;
        fre += fp_exact<D>(c) * pr;
        fim += fp_exact<D>(c) * pi;
      }
      prev = z;
    }
    acc[0] += (double)V[p] * n;
    acc[1] += n * n;
    acc[2] += fre * fre + fim * fim + fz * fz;
    acc[3] += n * n * sqrt(n);
  }
  block_reduce_store<4>(acc, partials, false);
}

// Sum over points of |A00|^2 = |sum_c (-1)^c psi_c psi_(D-1-c)|^2 / D, in FP64, for the
// nematic energy (c2/2) sum |A00|^2 dV (src/energy.jl:106-109, src/observables.jl:94-111).
template <typename R, int D>
__global__ void __launch_bounds__(kRedThreads) k_pair_energy(const cplx<R>* __restrict__ psi, int64_t N,
                                                             double* partials) {
  double acc[1] = {0.0};
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < N; p += (int64_t)gridDim.x * blockDim.x) {
    double ar = 0.0, ai = 0.0;
#pragma unroll
    for (int c = 0; c < D; ++c) {
      const cplx<R> x = psi[c * N + p], y = psi[(D - 1 - c) * N + p];
      const double pr = (double)x.x * y.x - (double)x.y * y.y;
      const double pi = (double)x.x * y.y + (double)x.y * y.x;
      ar += (c & 1) ? -pr : pr;
      ai += (c & 1) ? -pi : pi;
    }
    acc[0] += (ar * ar + ai * ai) / (double)D;
  }
  block_reduce_store<1>(acc, partials, false);
}

// Tensor energy sum_S g_S sum_M |A_SM|^2 (src/tensor_interaction.jl:247-276).
// Pair table rows: (a_idx, c1, c2) packed into int4 .x/.y/.z, coefficient cg*... in pcg.
template <typename R, int D>
__global__ void __launch_bounds__(kRedThreads) k_tensor_energy(const cplx<R>* __restrict__ psi, int64_t N,
                                                               const int4* __restrict__ pairs,
                                                               const double* __restrict__ pcg, int n_pairs,
                                                               const double* __restrict__ gA, int nA,
                                                               double* partials) {
  double acc[1] = {0.0};
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < N; p += (int64_t)gridDim.x * blockDim.x) {
    double2 v[D];
#pragma unroll
    for (int c = 0; c < D; ++c) {
      const cplx<R> z = psi[c * N + p];
      v[c] = make_double2((double)z.x, (double)z.y);
    }
    double e = 0.0;
    int cur = -1;
    double2 A = make_double2(0.0, 0.0);
    for (int q = 0; q < n_pairs; ++q) {
      const int4 pr = __ldg(pairs + q);
      if (pr.x != cur) {
        if (cur >= 0) e += 0.5 * gA[cur] * (A.x * A.x + A.y * A.y);
        cur = pr.x;
        A = make_double2(0.0, 0.0);
      }
      const double cg = __ldg(pcg + q);
      const double2 a = v[pr.y], b = v[pr.z];
      A.x += cg * (a.x * b.x - a.y * b.y);
      A.y += cg * (a.x * b.y + a.y * b.x);
    }
    if (cur >= 0) e += 0.5 * gA[cur] * (A.x * A.x + A.y * A.y);
    acc[0] += e;
    (void)nA;
  }
  block_reduce_store<1>(acc, partials, false);
}

// Order parameters of classify_phase (src/diagnostics.jl:166-206) as grid sums in FP64:
// out[0] = sum n, [1] = sum n^2, [2] = sum |<F>|^2, [3] = sum_m m |psi_m|^2 and
// [4 + S/2] = sum_M sum_x |A_SM|^2 for every even S <= 2F (pair_amplitude_spectrum,
// src/observables.jl:118-142,227-246).  Pair table rows (S/2, a = (S,M) index, c1, c2)
// sorted by a, with CG(F,m1;F,m2|S,M) in pcg (|CG| < 1e-15 dropped).
template <typename R, int D>
__global__ void __launch_bounds__(kRedThreads) k_phase_sums(const cplx<R>* __restrict__ psi, int64_t N,
                                                            SpinTabs<R> st, const int4* __restrict__ pairs,
                                                            const double* __restrict__ pcg, int n_pairs,
                                                            double* partials) {
  double acc[kPhaseSums];
#pragma unroll
  for (int k = 0; k < kPhaseSums; ++k) acc[k] = 0.0;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < N; p += (int64_t)gridDim.x * blockDim.x) {
    double2 v[D];
    double n = 0.0, fz = 0.0, fre = 0.0, fim = 0.0;
#pragma unroll
    for (int c = 0; c < D; ++c) {
      const cplx<R> z = psi[c * N + p];
      v[c] = make_double2((double)z.x, (double)z.y);
      const double a2 = v[c].x * v[c].x + v[c].y * v[c].y;
      n += a2;
      fz += (double)st.m[c] * a2;
      if (c >= 1) {
        fre += fp_exact<D>(c) * (v[c - 1].x * v[c].x + v[c - 1].y * v[c].y);
        fim += fp_exact<D>(c) * (v[c - 1].x * v[c].y - v[c - 1].y * v[c].x);
      }
    }
    acc[0] += n;
    acc[1] += n * n;
    acc[2] += fre * fre + fim * fim + fz * fz;
    acc[3] += fz;
    int cur = -1, cur_s = 0;
    double2 A = make_double2(0.0, 0.0);
    double w[kPhaseSums - 4];
#pragma unroll
    for (int s = 0; s < kPhaseSums - 4; ++s) w[s] = 0.0;
    for (int q = 0; q < n_pairs; ++q) {
      const int4 pr = __ldg(pairs + q);
      if (pr.y != cur) {
        if (cur >= 0) {
#pragma unroll
          for (int s = 0; s < kPhaseSums - 4; ++s)
            if (s == cur_s) w[s] += A.x * A.x + A.y * A.y;
        }
        cur = pr.y;
        cur_s = pr.x;
        A = make_double2(0.0, 0.0);
      }
      const double cg = __ldg(pcg + q);
      const double2 a = v[pr.z], b = v[pr.w];
      A.x += cg * (a.x * b.x - a.y * b.y);
      A.y += cg * (a.x * b.y + a.y * b.x);
    }
    if (cur >= 0) {
#pragma unroll
      for (int s = 0; s < kPhaseSums - 4; ++s)
        if (s == cur_s) w[s] += A.x * A.x + A.y * A.y;
    }
#pragma unroll
    for (int s = 0; s < kPhaseSums - 4; ++s) acc[4 + s] += w[s];
  }
  block_reduce_store<kPhaseSums>(acc, partials, false);
}

// Raman energy sum_x Re(psi^dagger H_R psi) = sum_x b(x)·<F>(x) (src/energy.jl:123-135), FP64.
template <typename R, int D>
__global__ void __launch_bounds__(kRedThreads) k_raman_energy(const cplx<R>* __restrict__ psi, int64_t N,
                                                              SpinTabs<R> st, RamanGeom g, double* partials) {
  double acc[1] = {0.0};
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < N; p += (int64_t)gridDim.x * blockDim.x) {
    double fz = 0.0, fre = 0.0, fim = 0.0;
    double2 prev = make_double2(0.0, 0.0);
#pragma unroll
    for (int c = 0; c < D; ++c) {
      const cplx<R> z0 = psi[c * N + p];
      const double2 z = make_double2((double)z0.x, (double)z0.y);
      fz += (double)st.m[c] * (z.x * z.x + z.y * z.y);
      if (c >= 1) {
        fre += fp_exact<D>(c) * (prev.x * z.x + prev.y * z.y);
        fim += fp_exact<D>(c) * (prev.x * z.y - prev.y * z.x);
      }
      prev = z;
    }
    double bx, by, bz;
    raman_field(g, p, bx, by, bz);
    acc[0] += bx * fre + by * fim + bz * fz;
  }
  block_reduce_store<1>(acc, partials, false);
}

// Kinetic energy sum_k k^2 |psi_hat_c(k)|^2 over all components of a transformed buffer.
template <typename R>
__global__ void __launch_bounds__(kRedThreads) k_kinetic_sum(const cplx<R>* __restrict__ a, int64_t N, int D,
                                                             PhaseTableArgs g, double* partials) {
  double acc[1] = {0.0};
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < N * D; q += (int64_t)gridDim.x * blockDim.x) {
    int64_t p = q % N;
    double k2 = 0.0;
    for (int ax = 0; ax < g.ndim; ++ax) {
      const int n = g.n[ax];
      const int m = (int)(p % n);
      p /= n;
      const double k = (double)freq_index(m, n) * g.kmult[ax];
      k2 += k * k;
    }
    const cplx<R> z = a[q];
    acc[0] += k2 * ((double)z.x * z.x + (double)z.y * z.y);
  }
  block_reduce_store<1>(acc, partials, false);
}

// sum Φ·F over the grid (src/energy.jl:111-121).
template <typename R>
__global__ void __launch_bounds__(kRedThreads) k_dot3(const R* __restrict__ a, const R* __restrict__ b, int64_t N,
                                                      double* partials) {
  double acc[1] = {0.0};
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < N; p += (int64_t)gridDim.x * blockDim.x) {
    acc[0] += (double)a[p] * b[p] + (double)a[N + p] * b[N + p] + (double)a[2 * N + p] * b[2 * N + p];
  }
  block_reduce_store<1>(acc, partials, false);
}

// [sum |a-b|^2, sum |b|^2] (src/adaptive.jl:42-50).
template <typename R>
__global__ void __launch_bounds__(kRedThreads) k_l2_change(const cplx<R>* __restrict__ a, const cplx<R>* __restrict__ b,
                                                           int64_t n, double* partials) {
  double acc[2] = {0.0, 0.0};
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    const cplx<R> x = a[q], y = b[q];
    const double dr = (double)x.x - (double)y.x, di = (double)x.y - (double)y.y;
    acc[0] += dr * dr + di * di;
    acc[1] += (double)y.x * y.x + (double)y.y * y.y;
  }
  block_reduce_store<2>(acc, partials, false);
}

// [max |a|, max |a-b|] (src/ground_state.jl:148-150); b may be null.
template <typename R>
__global__ void __launch_bounds__(kRedThreads) k_max_abs(const cplx<R>* __restrict__ a, const cplx<R>* __restrict__ b,
                                                         int64_t n, double* partials) {
  double acc[2] = {0.0, 0.0};
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    const cplx<R> x = a[q];
    acc[0] = fmax(acc[0], hypot((double)x.x, (double)x.y));
    if (b) {
      const cplx<R> y = b[q];
      acc[1] = fmax(acc[1], hypot((double)x.x - (double)y.x, (double)x.y - (double)y.y));
    }
  }
  block_reduce_store<2>(acc, partials, true);
}

// max |Φ| over the 3 DDI fields (src/ground_state.jl:12-17).
template <typename R>
__global__ void __launch_bounds__(kRedThreads) k_max_abs_real(const R* __restrict__ a, int64_t n, double* partials) {
  double acc[1] = {0.0};
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
    acc[0] = fmax(acc[0], fabs((double)a[q]));
  block_reduce_store<1>(acc, partials, true);
}

// ---------------------------------------------------------------------------
// Batched-solve reductions: grid (blocks per solve, active slots); per-block
// partials [slot][blk][K], then a per-solve fixed-order finish into out[solve][K].
// ---------------------------------------------------------------------------
template <int K>
__device__ __forceinline__ void block_reduce_store_2d(double (&vals)[K], double* partials, bool is_max) {
  __shared__ double red[K][kRedThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    double x = vals[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double y = __shfl_down_sync(0xffffffffu, x, o);
      x = is_max ? fmax(x, y) : x + y;
    }
    if (lane == 0) red[k][warp] = x;
  }
  __syncthreads();
  if (threadIdx.x < K) {
    const int k = threadIdx.x;
    double x = red[k][0];
    for (int w = 1; w < kRedThreads / 32; ++w) x = is_max ? fmax(x, red[k][w]) : x + red[k][w];
    partials[((size_t)blockIdx.y * gridDim.x + blockIdx.x) * K + k] = x;
  }
}

template <int K>
__global__ void k_seg_finish(const double* __restrict__ partials, int nb, int n_slots, const int* __restrict__ active,
                             int is_max, double* __restrict__ out, int out_stride) {
  const int slot = blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= n_slots) return;
  const int b = active ? active[slot] : slot;
  for (int k = 0; k < K; ++k) {
    double x = 0.0;
    for (int i = 0; i < nb; ++i) {
      const double y = partials[((size_t)slot * nb + i) * K + k];
      x = is_max ? fmax(x, y) : x + y;
    }
    out[(size_t)b * out_stride + k] = x;
  }
}

// Row-pass norm partials: one per block, blocks grouped by slot.
template <typename R>
__global__ void k_seg_finish_rows(const double* __restrict__ partials, int bps, int n_slots,
                                  const int* __restrict__ active, double* __restrict__ out) {
  pdl_wait();
  const int slot = blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= n_slots) return;
  double x = 0.0;
  for (int i = 0; i < bps; ++i) x += partials[(size_t)slot * bps + i];
  out[active ? active[slot] : slot] = x;
}

// Batched ITP with a predicted renormalisation (RP_MID): from the norm partials of
// each active solve, the actual scale s = 1/sqrt(norm dV), the correction
// corr = s / pred for the next pass's load, and the next prediction pred = s.
template <typename R>
__global__ void k_seg_pred(const double* __restrict__ partials, int bps, int n_slots, const int* __restrict__ active,
                           double dV, R* __restrict__ corr, R* __restrict__ pred) {
  pdl_wait();
  const int slot = blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= n_slots) return;
  double x = 0.0;
  for (int i = 0; i < bps; ++i) x += partials[(size_t)slot * bps + i];
  const int b = active[slot];
  const double sc = 1.0 / sqrt(x * dV);
  corr[b] = (R)(sc / (double)pred[b]);
  pred[b] = (R)sc;
}

// Per-solve [sum n^2... ] energy terms and component sums: K = D + 4 values
// [comp sums(D), trap, n^2, |f|^2, n^{5/2}] for solve active[blockIdx.y].
template <typename R, int D>
__global__ void __launch_bounds__(kRedThreads) k_batch_energy_local(const cplx<R>* __restrict__ psi, int64_t N,
                                                                    int64_t solve_stride,
                                                                    const int* __restrict__ active,
                                                                    const R* __restrict__ V, SpinTabs<R> st,
                                                                    double* partials) {
  double acc[D + 4];
#pragma unroll
  for (int k = 0; k < D + 4; ++k) acc[k] = 0.0;
  const cplx<R>* base = psi + (int64_t)active[blockIdx.y] * solve_stride;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < N; p += (int64_t)gridDim.x * blockDim.x) {
    double n = 0.0, fz = 0.0, fre = 0.0, fim = 0.0;
    cplx<R> prev = mk<R>(0, 0);
#pragma unroll
    for (int c = 0; c < D; ++c) {
      const cplx<R> z = base[c * N + p];
      const double a2 = (double)z.x * z.x + (double)z.y * z.y;
      acc[c] += a2;
      n += a2;
      fz += (double)st.m[c] * a2;
      if (c >= 1) {
        fre += fp_exact<D>(c) * ((double)prev.x * z.x + (double)prev.y * z.y);
        fim += fp_exact<D>(c) * ((double)prev.x * z.y - (double)prev.y * z.x);
      }
      prev = z;
    }
    acc[D] += (double)V[p] * n;
    acc[D + 1] += n * n;
    acc[D + 2] += fre * fre + fim * fim + fz * fz;
    acc[D + 3] += n * n * sqrt(n);
  }
  block_reduce_store_2d<D + 4>(acc, partials, false);
}

// Per-solve sum over points of |A00|^2 (the nematic energy, as k_pair_energy) for solve
// active[blockIdx.y].
template <typename R, int D>
__global__ void __launch_bounds__(kRedThreads) k_batch_pair_energy(const cplx<R>* __restrict__ psi, int64_t N,
                                                                   int64_t solve_stride,
                                                                   const int* __restrict__ active,
                                                                   double* partials) {
  double acc[1] = {0.0};
  const cplx<R>* base = psi + (int64_t)active[blockIdx.y] * solve_stride;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < N; p += (int64_t)gridDim.x * blockDim.x) {
    double ar = 0.0, ai = 0.0;
#pragma unroll
    for (int c = 0; c < D; ++c) {
      const cplx<R> x = base[c * N + p], y = base[(D - 1 - c) * N + p];
      const double pr = (double)x.x * y.x - (double)x.y * y.y;
      const double pi = (double)x.x * y.y + (double)x.y * y.x;
      ar += (c & 1) ? -pr : pr;
      ai += (c & 1) ? -pi : pi;
    }
    acc[0] += (ar * ar + ai * ai) / (double)D;
  }
  block_reduce_store_2d<1>(acc, partials, false);
}

// Per-solve kinetic sum over a compact (slot-ordered) transformed scratch buffer.
template <typename R>
__global__ void __launch_bounds__(kRedThreads) k_batch_kinetic_sum(const cplx<R>* __restrict__ a, int64_t N, int D,
                                                                   PhaseTableArgs g, double* partials) {
  double acc[1] = {0.0};
  const cplx<R>* base = a + (int64_t)blockIdx.y * N * D;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < N * D; q += (int64_t)gridDim.x * blockDim.x) {
    int64_t p = q % N;
    double k2 = 0.0;
    for (int ax = 0; ax < g.ndim; ++ax) {
      const int n = g.n[ax];
      const int m = (int)(p % n);
      p /= n;
      const double k = (double)freq_index(m, n) * g.kmult[ax];
      k2 += k * k;
    }
    const cplx<R> z = base[q];
    acc[0] += k2 * ((double)z.x * z.x + (double)z.y * z.y);
  }
  block_reduce_store_2d<1>(acc, partials, false);
}

// Per-solve [max |psi|, max |psi - prev|].
template <typename R>
__global__ void __launch_bounds__(kRedThreads) k_batch_max_abs(const cplx<R>* __restrict__ a,
                                                               const cplx<R>* __restrict__ b, int64_t n,
                                                               int64_t solve_stride, const int* __restrict__ active,
                                                               double* partials) {
  double acc[2] = {0.0, 0.0};
  const int64_t off = (int64_t)active[blockIdx.y] * solve_stride;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    const cplx<R> x = a[off + q], y = b[off + q];
    acc[0] = fmax(acc[0], hypot((double)x.x, (double)x.y));
    acc[1] = fmax(acc[1], hypot((double)x.x - (double)y.x, (double)x.y - (double)y.y));
  }
  block_reduce_store_2d<2>(acc, partials, true);
}

// Copy the active solves (slot order) between a strided batch buffer and a compact one.
template <typename R>
__global__ void k_batch_gather(const cplx<R>* __restrict__ src, cplx<R>* __restrict__ dst, int64_t per_solve,
                               const int* __restrict__ active, int n_slots, int to_compact) {
  const int64_t total = per_solve * n_slots;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
    const int slot = (int)(q / per_solve);
    const int64_t r = q % per_solve;
    const int64_t sidx = (int64_t)active[slot] * per_solve + r;
    if (to_compact) dst[q] = src[sidx];
    else dst[sidx] = src[q];
  }
}

// ---------------------------------------------------------------------------
// Elementwise helpers
// ---------------------------------------------------------------------------
template <typename R>
__global__ void k_scale(cplx<R>* a, int64_t n, double s) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
    a[q] = a[q] * (R)s;
}

// psi /= sqrt(sum_c sums[c]*dV) with the sums already on the device (src/split_step.jl:185-195).
template <typename R>
__global__ void k_normalize_apply(cplx<R>* a, int64_t N, int D, const double* __restrict__ sums, double dV) {
  pdl_wait();
  double ns = 0.0;
  for (int c = 0; c < D; ++c) ns += sums[c] * dV;
  const R s = (R)(1.0 / sqrt(ns));
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < N * D; q += (int64_t)gridDim.x * blockDim.x)
    a[q] = a[q] * s;
}

// psi_b /= sqrt(norm[b]*dV) for the active solves of a batch.
template <typename R>
__global__ void k_batch_normalize(cplx<R>* a, int64_t per_solve, const int* __restrict__ active, int n_slots,
                                  const double* __restrict__ norm, double dV) {
  pdl_wait();
  const int64_t total = per_solve * n_slots;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
    const int b = active[q / per_solve];
    const R s = (R)(1.0 / sqrt(norm[b] * dV));
    a[(int64_t)b * per_solve + q % per_solve] = a[(int64_t)b * per_solve + q % per_solve] * s;
  }
}

// Per-component scale psi_c *= w[c] (constrained normalisation, src/ground_state.jl:312-317).
template <typename R>
__global__ void k_scale_comp(cplx<R>* a, int64_t N, int D, const double* w) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < N * D; q += (int64_t)gridDim.x * blockDim.x)
    a[q] = a[q] * (R)w[q / N];
}

template <typename R>
__global__ void k_from_f64(const double2* __restrict__ src, cplx<R>* __restrict__ dst, int64_t n) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
    dst[q] = mk<R>((R)src[q].x, (R)src[q].y);
}

template <typename R>
__global__ void k_to_f64(const cplx<R>* __restrict__ src, double2* __restrict__ dst, int64_t n) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
    dst[q] = make_double2((double)src[q].x, (double)src[q].y);
}

template <typename R>
__global__ void k_real_from_f64(const double* __restrict__ src, R* __restrict__ dst, int64_t n) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
    dst[q] = (R)src[q];
}

template <typename R>
__global__ void k_real_to_f64(const R* __restrict__ src, double* __restrict__ dst, int64_t n) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
    dst[q] = (double)src[q];
}

}  // namespace sbec
