// Native FP64 instantiation of the engine.
#include "engine_impl.cuh"
namespace laps {
template class Engine<double>;
EngineBase* make_engine_fp64(const laps_params& p) { return new Engine<double>(p); }
long long plan_bytes_fp64(const laps_params& p) { return Engine<double>::plan_bytes(p); }
}  // namespace laps
