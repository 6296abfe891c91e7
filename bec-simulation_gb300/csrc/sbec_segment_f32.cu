// Persistent 2-D leapfrog segments (FP32): the cooperative launch of k_lf_segment.
#include <mutex>

#include "sbec_lines_impl.cuh"

namespace sbec {

namespace {

template <int NN, int D>
void seg_launch(const LineCtx<float>& c, const Tw<float>& twx, const Tw<float>& twy, const RowArgs<float>& a,
                long long n_steps, GridBarrier* bar) {
  using Sh = SegShape<float, NN, NN, D, 0>;
  auto kern = k_lf_segment<float, NN, NN, D, 0>;
  // resident blocks of the whole GPU: a cooperative launch may not exceed them.  The
  // shared-memory attribute and the occupancy are per device, so they are kept per device
  // ordinal and set up the first time a segment runs on that device.
  constexpr int kMaxDev = 64;
  static std::mutex mu;
  static int resident_of[kMaxDev] = {};
  int dev = 0;
  cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDev) fail(SBEC_ERR_UNSUPPORTED, "device ordinal beyond the segment table");
  int resident = 0;
  {
    std::lock_guard<std::mutex> lock(mu);
    if (resident_of[dev] == 0) {
      line_set_smem(kern, Sh::smem_bytes);
      int sms = 0, occ = 0;
      cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "cudaDeviceGetAttribute");
      cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, Sh::T, Sh::smem_bytes),
                 "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
      resident_of[dev] = std::max(sms * occ, -1);
      if (resident_of[dev] == 0) resident_of[dev] = -1;
    }
    resident = resident_of[dev];
  }
  if (resident < 1) fail(SBEC_ERR_UNSUPPORTED, "segment kernel does not fit on an SM");
  const int row_units = (int)((a.n_rows + Sh::RPB - 1) / Sh::RPB);
  const int col_units = (NN + Sh::W - 1) / Sh::W * D;
  const int blocks = std::min(resident, std::max(row_units, col_units));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)blocks);
  cfg.blockDim = dim3(Sh::T);
  cfg.dynamicSmemBytes = Sh::smem_bytes;
  cfg.stream = c.stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cuda_check(cudaLaunchKernelEx(&cfg, kern, a, c.st, c.ph, twx, twy, n_steps, bar), "cooperative segment launch");
}

template <int NN>
void seg_launch_d(const LineCtx<float>& c, const Tw<float>& twx, const Tw<float>& twy, const RowArgs<float>& a, int D,
                  long long n_steps, GridBarrier* bar) {
  if (D == 1) seg_launch<NN, 1>(c, twx, twy, a, n_steps, bar);
  else if (D == 3) seg_launch<NN, 3>(c, twx, twy, a, n_steps, bar);
  else fail(SBEC_ERR_UNSUPPORTED, "segment kernel needs D in {1,3}");
}

}  // namespace

bool lf_segment_supported(bool fp32, int nx, int ny, int D) {
  return fp32 && nx == ny && (nx == 64 || nx == 128 || nx == 256 || nx == 512) && (D == 1 || D == 3);
}

void lf_segment_launch(const LineCtx<float>& c, const Tw<float>& twx, const Tw<float>& twy, const RowArgs<float>& a,
                       int n, int D, long long n_steps, GridBarrier* bar) {
  switch (n) {
    case 64: seg_launch_d<64>(c, twx, twy, a, D, n_steps, bar); return;
    case 128: seg_launch_d<128>(c, twx, twy, a, D, n_steps, bar); return;
    case 256: seg_launch_d<256>(c, twx, twy, a, D, n_steps, bar); return;
    case 512: seg_launch_d<512>(c, twx, twy, a, D, n_steps, bar); return;
    default: fail(SBEC_ERR_UNSUPPORTED, "segment kernel: unsupported grid " + std::to_string(n));
  }
}

}  // namespace sbec
