// Shared device helpers: complex arithmetic on double2 / float2, precision traits.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace sbec {

template <typename R> struct CplxOf;
template <> struct CplxOf<double> { using type = double2; };
template <> struct CplxOf<float> { using type = float2; };
template <typename R> using cplx = typename CplxOf<R>::type;

template <typename R>
__host__ __device__ __forceinline__ cplx<R> mk(R re, R im) {
  cplx<R> z;
  z.x = re;
  z.y = im;
  return z;
}

#define SBEC_CPLX_OPS(T2, R)                                                                      \
  __host__ __device__ __forceinline__ T2 operator+(T2 a, T2 b) { return mk<R>(a.x + b.x, a.y + b.y); } \
  __host__ __device__ __forceinline__ T2 operator-(T2 a, T2 b) { return mk<R>(a.x - b.x, a.y - b.y); } \
  __host__ __device__ __forceinline__ T2 operator-(T2 a) { return mk<R>(-a.x, -a.y); }           \
  __host__ __device__ __forceinline__ T2 operator*(T2 a, T2 b) {                                 \
    return mk<R>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);                                   \
  }                                                                                               \
  __host__ __device__ __forceinline__ T2 operator*(R s, T2 a) { return mk<R>(s * a.x, s * a.y); } \
  __host__ __device__ __forceinline__ T2 operator*(T2 a, R s) { return mk<R>(a.x * s, a.y * s); } \
  __host__ __device__ __forceinline__ T2& operator+=(T2& a, T2 b) {                              \
    a.x += b.x;                                                                                   \
    a.y += b.y;                                                                                   \
    return a;                                                                                     \
  }                                                                                               \
  __host__ __device__ __forceinline__ T2& operator-=(T2& a, T2 b) {                              \
    a.x -= b.x;                                                                                   \
    a.y -= b.y;                                                                                   \
    return a;                                                                                     \
  }                                                                                               \
  __host__ __device__ __forceinline__ T2& operator*=(T2& a, T2 b) {                              \
    a = a * b;                                                                                    \
    return a;                                                                                     \
  }                                                                                               \
  __host__ __device__ __forceinline__ T2& operator*=(T2& a, R s) {                               \
    a.x *= s;                                                                                     \
    a.y *= s;                                                                                     \
    return a;                                                                                     \
  }                                                                                               \
  __host__ __device__ __forceinline__ T2 conj(T2 a) { return mk<R>(a.x, -a.y); }                \
  __host__ __device__ __forceinline__ R abs2(T2 a) { return a.x * a.x + a.y * a.y; }             \
  /* conj(a) * b */                                                                               \
  __host__ __device__ __forceinline__ T2 cmulc(T2 a, T2 b) {                                     \
    return mk<R>(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);                                   \
  }                                                                                               \
  /* i * a */                                                                                     \
  __host__ __device__ __forceinline__ T2 mul_i(T2 a) { return mk<R>(-a.y, a.x); }               \
  /* -i * a */                                                                                    \
  __host__ __device__ __forceinline__ T2 mul_mi(T2 a) { return mk<R>(a.y, -a.x); }

SBEC_CPLX_OPS(double2, double)
SBEC_CPLX_OPS(float2, float)
#undef SBEC_CPLX_OPS

// cis(x) = cos(x) + i sin(x), in the working precision.
__device__ __forceinline__ double2 cis_(double x) {
  double s, c;
  sincos(x, &s, &c);
  return mk<double>(c, s);
}
__device__ __forceinline__ float2 cis_(float x) {
  float s, c;
  sincosf(x, &s, &c);
  return mk<float>(c, s);
}

// x * (wh + wl) where wh + wl is a unit complex number split into a float head
// and tail: the tail term removes the systematic magnitude error of the rounded
// head, so FP32 products with fixed twiddles / phases round without bias.
__device__ __forceinline__ float2 cmul_comp(float2 x, float2 wh, float2 wl) {
  const float sr = fmaf(x.x, wl.x, -x.y * wl.y);
  const float si = fmaf(x.x, wl.y, x.y * wl.x);
  return mk<float>(fmaf(x.x, wh.x, fmaf(-x.y, wh.y, sr)), fmaf(x.x, wh.y, fmaf(x.y, wh.x, si)));
}
__device__ __forceinline__ double2 cmul_comp(double2 x, double2 wh, double2) { return x * wh; }

// Twiddle / phase table: head values; FP32 tables store (head, tail) pairs
// interleaved, entry e at hi[2e], hi[2e+1].
template <typename R>
struct Tw {
  const cplx<R>* hi;
  const cplx<R>* lo;
};

// x * w (or conj w) for a table twiddle.  FP32 tables interleave head and tail
// (one 16-byte load) and use the compensated product.
template <typename R>
__device__ __forceinline__ cplx<R> tw_mul(cplx<R> x, const Tw<R>& t, int idx, bool conj_w) {
  if constexpr (sizeof(R) == 4) {
    const float4 w4 = __ldg(reinterpret_cast<const float4*>(t.hi) + idx);
    float2 wh = mk<float>(w4.x, w4.y), wl = mk<float>(w4.z, w4.w);
    if (conj_w) {
      wh.y = -wh.y;
      wl.y = -wl.y;
    }
    return cmul_comp(x, wh, wl);
  } else {
    cplx<R> w = __ldg(t.hi + idx);
    if (conj_w) w.y = -w.y;
    return x * w;
  }
}

// a + b rounded to FP32 without a systematic bias, for |a| >= |b| (a state value plus
// a small correction).  The exact sum is s + e (Fast2Sum); s moves one ulp towards e
// when |e| exceeds a threshold drawn uniformly from [0, ulp) by a hash of the operands'
// bits (deterministic: equal inputs give equal results), so the expected result is
// the exact sum.  Needed where an FP32 state is turned by small angles near a
// coordinate axis: near the real axis the inward shift of the real part (x^2/2 |z|) is
// below half an ulp and round-to-nearest keeps it outside every time while the
// imaginary part, near zero, is resolved finely — a slowly turning near-real state (the
// polar ground state in its trap, or its real spectrum under the kinetic phase) then
// gains norm at x^2 per rotation.
__device__ __forceinline__ float sr_add(float a, float b, unsigned salt) {
  const float s = __fadd_rn(a, b);
  const float e = __fsub_rn(b, __fsub_rn(s, a));
  const float up = __int_as_float(__float_as_int(s) + (((e > 0.0f) == (s > 0.0f)) ? 1 : -1));
  const unsigned h = (__float_as_uint(a) ^ (__float_as_uint(b) * 0x9E3779B9u) ^ salt) >> 8;
  const float thr = (float)h * (1.0f / 16777216.0f) * fabsf(up - s);
  return (e != 0.0f && s != 0.0f && fabsf(e) > thr) ? up : s;
}

// x * w for a kinetic phase table entry.  Real-time FP32 tables hold
// scale * (cos, sin) as (head, tail) with scale an exact power of two (1/N on the x
// axis, where the inverse-FFT normalisation is folded in, 1 elsewhere); the product is
// formed as x scale + x (w - scale): x scale is exact, w - scale comes from the head and
// tail without cancellation for the small angles of low k, and the final addition is
// rounded without bias (sr_add) — a near-real spectrum turned by small angles would
// otherwise gain norm at every step.  Imaginary-time (decay) tables, renormalised every
// step, and FP64 use the compensated / plain product.
template <typename R>
__device__ __forceinline__ cplx<R> phase_mul(cplx<R> x, const Tw<R>& t, int idx, R scale, int unbiased) {
  if constexpr (sizeof(R) == 4) {
    const float4 w4 = __ldg(reinterpret_cast<const float4*>(t.hi) + idx);
    if (!unbiased) return cmul_comp(x, mk<float>(w4.x, w4.y), mk<float>(w4.z, w4.w));
    const float cm = __fadd_rn(__fsub_rn(w4.x, scale), w4.z);
    const float sn = __fadd_rn(w4.y, w4.w);
    const float bx = __fmaf_rn(x.x, cm, __fmul_rn(-x.y, sn));
    const float by = __fmaf_rn(x.y, cm, __fmul_rn(x.x, sn));
    return mk<float>(sr_add(__fmul_rn(x.x, scale), bx, 0x85ebca6bu), sr_add(__fmul_rn(x.y, scale), by, 0xc2b2ae35u));
  } else {
    (void)scale;
    (void)unbiased;
    return x * __ldg(t.hi + idx);
  }
}

template <typename R>
__device__ __forceinline__ cplx<R> ldg(const cplx<R>* p) {
  return __ldg(p);
}

template <typename R>
__device__ __forceinline__ R ldg_r(const R* p) {
  return __ldg(p);
}

// Programmatic dependent launch (both are no-ops for a launch without the attribute).
// pdl_wait: at kernel start, wait until the previous grid has completed and its
// writes are visible.  pdl_trigger: late in a kernel, let the next grid start
// launching (its blocks then wait in pdl_wait); placed before the final stores so the
// next grid's launch overlaps this grid's tail instead of holding SM slots for the
// whole of this grid.
__device__ __forceinline__ void pdl_wait() {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 900
  cudaGridDependencySynchronize();
#endif
}
__device__ __forceinline__ void pdl_trigger() {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 900
  cudaTriggerProgrammaticLaunchCompletion();
#endif
}

constexpr int kMaxD = 13;      // F <= 6
constexpr int kMaxAxis = 3;

}  // namespace sbec
