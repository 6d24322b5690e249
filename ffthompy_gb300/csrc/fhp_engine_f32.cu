// Engine instantiation: single precision fields/FFT with FP64 reductions.
#include "fhp_engine_impl.cuh"

namespace fhp {
std::unique_ptr<EngineBase> make_engine_f32(const PlanConfig& cfg, int* status) {
  auto e = std::make_unique<Engine<float>>(cfg);
  *status = e->init();
  if (*status != ST_OK) return nullptr;
  return e;
}
}  // namespace fhp
