// Float-float instantiation of the engine.
#include "engine_impl.cuh"
namespace laps {
template class Engine<dd>;
EngineBase* make_engine_dd(const laps_params& p) { return new Engine<dd>(p); }
long long plan_bytes_dd(const laps_params& p) { return Engine<dd>::plan_bytes(p); }
}  // namespace laps
