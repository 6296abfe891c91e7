// Measured FMA throughput of the current device, the denominators of the compute rooflines
// (the FP64-pipe-bound plain form, the FP32 tensor step).  Each thread runs eight independent
// chains x <- fma(x, a, b) in registers; a and b arrive as kernel arguments, so nothing folds
// at compile time, and a ~ 1, b small keep every value normal.  No counterpart in the
// reference.
#include <cuda_runtime.h>

#include <string>

#include "sbec.h"
#include "sbec_engine.h"
#include "sbec_setup.h"

namespace sbec {
namespace {

constexpr int kPeakThreads = 256;
constexpr int kPeakChains = 8;

template <typename T>
__global__ void __launch_bounds__(kPeakThreads) k_fma_peak(T* out, int iters, T a, T b) {
  T x[kPeakChains];
#pragma unroll
  for (int k = 0; k < kPeakChains; ++k) x[k] = (T)(threadIdx.x + k) * (T)1e-3;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < kPeakChains; ++k) x[k] = fma(x[k], a, b);
  }
  T s = 0;
#pragma unroll
  for (int k = 0; k < kPeakChains; ++k) s += x[k];
  if (s == (T)-1.2345) out[0] = s;  // keeps the chains live; never true for these inputs
}

template <typename T>
double measure(int iters) {
  int dev = 0, sms = 0;
  cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "cudaDeviceGetAttribute");
  T* out = nullptr;
  cuda_check(cudaMalloc(&out, sizeof(T)), "cudaMalloc");
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaStream_t st = nullptr;
  double best = 0.0;
  try {
    cuda_check(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate");
    cuda_check(cudaEventCreate(&e0), "cudaEventCreate");
    cuda_check(cudaEventCreate(&e1), "cudaEventCreate");
    const int blocks = sms * 8;  // 2048 threads per SM
    const T a = (T)0.999999, b = (T)1e-6;
    k_fma_peak<T><<<blocks, kPeakThreads, 0, st>>>(out, iters / 8, a, b);  // warm-up
    cuda_check(cudaGetLastError(), "k_fma_peak");
    for (int rep = 0; rep < 3; ++rep) {
      cuda_check(cudaEventRecord(e0, st), "cudaEventRecord");
      k_fma_peak<T><<<blocks, kPeakThreads, 0, st>>>(out, iters, a, b);
      cuda_check(cudaGetLastError(), "k_fma_peak");
      cuda_check(cudaEventRecord(e1, st), "cudaEventRecord");
      cuda_check(cudaEventSynchronize(e1), "cudaEventSynchronize");
      float ms = 0.f;
      cuda_check(cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime");
      const double flops = 2.0 * kPeakChains * (double)iters * blocks * kPeakThreads;
      best = std::max(best, flops / (ms * 1e-3) / 1e12);
    }
  } catch (...) {
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st) cudaStreamDestroy(st);
    cudaFree(out);
    throw;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(st);
  cudaFree(out);
  return best;
}

}  // namespace
}  // namespace sbec

using namespace sbec;

extern "C" sbec_status sbec_measure_fma_peak(int32_t precision, double* tflops) {
  try {
    if (!tflops) fail(SBEC_ERR_INVALID, "tflops must not be NULL");
    if (sbec_device_count() < 1) fail(SBEC_ERR_DEVICE, "no CUDA device available");
    if (precision == SBEC_FP32_BULK)
      *tflops = measure<float>(1 << 16);
    else if (precision == SBEC_FP64)
      *tflops = measure<double>(1 << 12);
    else
      fail(SBEC_ERR_INVALID, "precision must be SBEC_FP64 or SBEC_FP32_BULK");
  } catch (const SbecError& e) {
    set_last_error(e.msg);
    return e.status;
  }
  return SBEC_OK;
}
