// FP32-bulk instantiation of the engine (reductions stay FP64).
#include "sbec_engine_impl.cuh"

namespace sbec {
std::unique_ptr<EngineBase> make_engine_f32(const Setup& s) { return std::make_unique<Engine<float>>(s); }

bool fused_path_supported(const Setup& s, bool fp32) {
  if (!s.pow2 || s.ddi || s.tensor || s.raman || s.loss) return false;
  if (!(s.D == 1 || s.D == 3 || s.D == 5)) return false;
  const int nx = s.n[0];
  if (nx < 16 || nx > 4096) return false;
  return row_variant_ok(fp32, nx, s.D, 0);
}
}  // namespace sbec
