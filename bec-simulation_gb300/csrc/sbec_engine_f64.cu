// FP64 (plain form) instantiation of the engine.
#include "sbec_engine_impl.cuh"

namespace sbec {
std::unique_ptr<EngineBase> make_engine_f64(const Setup& s) { return std::make_unique<Engine<double>>(s); }
}  // namespace sbec
