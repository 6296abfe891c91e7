// FP32-bulk instantiation of the engine (reductions stay FP64).
#include "sbec_engine_impl.cuh"

namespace sbec {
std::unique_ptr<EngineBase> make_engine_f32(const Setup& s) { return std::make_unique<Engine<float>>(s); }
}  // namespace sbec
