// Engine instantiation: double precision (the plain FP64 path).
#include "fhp_engine_impl.cuh"

namespace fhp {
std::unique_ptr<EngineBase> make_engine_f64(const PlanConfig& cfg, int* status) {
  auto e = std::make_unique<Engine<double>>(cfg);
  *status = e->init();
  if (*status != ST_OK) return nullptr;
  return e;
}
}  // namespace fhp
