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

template <typename R>
__device__ __forceinline__ cplx<R> ldg(const cplx<R>* p) {
  return __ldg(p);
}

template <typename R>
__device__ __forceinline__ R ldg_r(const R* p) {
  return __ldg(p);
}

constexpr int kMaxD = 13;      // F <= 6
constexpr int kMaxAxis = 3;

}  // namespace sbec
