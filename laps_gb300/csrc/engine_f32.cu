// FP32-transform instantiation of the engine: transforms and products in FP32, the state,
// the RK register, the CFL arithmetic and the diagnostics in float-float.
#include "engine_impl.cuh"
namespace laps {
template class Engine<float, dd>;
EngineBase* make_engine_f32(const laps_params& p) { return new Engine<float, dd>(p); }
long long plan_bytes_f32(const laps_params& p) { return Engine<float, dd>::plan_bytes(p); }
}  // namespace laps
