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
