// Allocation-free per-component norms of a caller-owned device wavefunction.
//
// Some callers of this library cannot allocate GPU memory when they need a
// reduction: code running while a CUDA stream is being captured into a graph
// (cudaMalloc/cudaFree are not capturable), and host programs whose GPU memory is
// owned by another allocator (a Julia CUDA.jl memory pool, a framework's caching
// allocator) that must not see driver allocations behind its back.  The
// workspace entry points allocate their reduction scratch when a workspace is
// created; this entry point instead keeps its scratch in a fixed file-scope
// device array, so a call allocates nothing.
//
// The scratch array is shared by every call on a device and keeps the previous
// call's contents.  Every call overwrites the whole region it reads, so nothing
// needs clearing, but two calls whose kernels overlap on the GPU (e.g. on two
// streams) race on it: serialise them.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <string>

#include "sbec.h"
#include "sbec_engine.h"
#include "sbec_setup.h"

namespace sbec {

namespace {

constexpr int kNaBlocks = 1024;              // reduction blocks per call
constexpr int kNaThreads = 256;
constexpr int kNaSlots = SBEC_NOALLOC_MAX_COMPONENTS + 1;  // D sums + NaN count
constexpr int kMaxDevices = 64;

// 1024 blocks x 32 slots x 8 bytes = 256 KiB per device, held until process exit.
static __device__ __align__(256) double g_noalloc_partials[kNaBlocks * 32];

struct DevScratch {
  double* ptr = nullptr;
  bool ready = false;
};
DevScratch g_dev[kMaxDevices];
std::mutex g_mu;

double* scratch_for_current_device() {
  int dev = 0;
  cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) fail(SBEC_ERR_UNSUPPORTED, "device ordinal beyond the no-alloc table");
  std::lock_guard<std::mutex> lock(g_mu);
  DevScratch& d = g_dev[dev];
  if (!d.ready) {
    // The host-side name of a __device__ array is a stand-in, not a device
    // address: resolve it once per device, with that device current.
    void* p = nullptr;
    cuda_check(cudaGetSymbolAddress(&p, g_noalloc_partials), "cudaGetSymbolAddress");
    d.ptr = static_cast<double*>(p);
    d.ready = true;
  }
  return d.ptr;
}

// Per-block partial sums of |psi_c|^2 for c < D, and the NaN count in slot D.
__global__ void __launch_bounds__(kNaThreads) k_na_partials(const double2* __restrict__ psi, int64_t n, int D,
                                                             double* __restrict__ part) {
  __shared__ double red[kNaSlots][kNaThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int c = 0; c <= D; ++c) {
    double acc = 0.0;
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
      if (c < D) {
        const double2 z = psi[(int64_t)c * n + p];
        acc += z.x * z.x + z.y * z.y;
      } else {
        for (int cc = 0; cc < D; ++cc) {
          const double2 z = psi[(int64_t)cc * n + p];
          if (isnan(z.x) || isnan(z.y)) acc += 1.0;
        }
      }
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) red[c][warp] = acc;
  }
  __syncthreads();
  if (threadIdx.x <= D) {
    double x = 0.0;
    for (int w = 0; w < kNaThreads / 32; ++w) x += red[threadIdx.x][w];
    part[(size_t)blockIdx.x * 32 + threadIdx.x] = x;
  }
}

// Fixed-order sum over the blocks into the caller's output.
__global__ void k_na_finish(const double* __restrict__ part, int nb, int D, double* __restrict__ out) {
  const int c = threadIdx.x;
  if (c > D) return;
  double x = 0.0;
  for (int b = 0; b < nb; ++b) x += part[(size_t)b * 32 + c];
  out[c] = x;
}

}  // namespace

}  // namespace sbec

using namespace sbec;

extern "C" sbec_status sbec_component_norms_noalloc(const double* psi_dev, int64_t n_points, int32_t n_components,
                                                    double* sums_dev, void* stream) {
  try {
    if (!psi_dev || !sums_dev) fail(SBEC_ERR_INVALID, "psi_dev and sums_dev must be device pointers, not NULL");
    if (n_points <= 0) fail(SBEC_ERR_INVALID, "n_points must be positive");
    if (n_components < 1 || n_components > SBEC_NOALLOC_MAX_COMPONENTS)
      fail(SBEC_ERR_INVALID, "n_components must be in 1.." + std::to_string(SBEC_NOALLOC_MAX_COMPONENTS) +
                                 " (the fixed scratch holds one slot per component)");
    if (n_points > SBEC_NOALLOC_MAX_POINTS)
      fail(SBEC_ERR_INVALID, "n_points exceeds SBEC_NOALLOC_MAX_POINTS (" + std::to_string(SBEC_NOALLOC_MAX_POINTS) + ")");
    // psi is read as complex doubles (16-byte loads); a view at an odd double offset would fault
    if ((reinterpret_cast<uintptr_t>(psi_dev) & 15) != 0)
      fail(SBEC_ERR_INVALID, "psi_dev must be 16-byte aligned (whole complex Float64 entries)");
    if ((reinterpret_cast<uintptr_t>(sums_dev) & 7) != 0) fail(SBEC_ERR_INVALID, "sums_dev must be 8-byte aligned");
    double* part = scratch_for_current_device();
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int64_t want = (n_points + kNaThreads - 1) / kNaThreads;
    const int nb = (int)(want < kNaBlocks ? want : kNaBlocks);
    k_na_partials<<<nb, kNaThreads, 0, st>>>(reinterpret_cast<const double2*>(psi_dev), n_points, n_components, part);
    cuda_check(cudaGetLastError(), "k_na_partials");
    k_na_finish<<<1, 32, 0, st>>>(part, nb, n_components, sums_dev);
    cuda_check(cudaGetLastError(), "k_na_finish");
  } catch (const SbecError& e) {
    set_last_error(e.msg);
    return e.status;
  }
  return SBEC_OK;
}
