// FP32-transform instantiation with an IEEE FP64 state: transforms and products in FP32,
// the state, the RK register, the CFL arithmetic and the diagnostics in FP64.
#include "engine_impl.cuh"
namespace laps {
template class Engine<float, double>;
EngineBase* make_engine_f32d(const laps_params& p) { return new Engine<float, double>(p); }
long long plan_bytes_f32d(const laps_params& p) { return Engine<float, double>::plan_bytes(p); }
}  // namespace laps
