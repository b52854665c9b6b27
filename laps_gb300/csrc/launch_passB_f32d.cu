// Pass B launcher (float transforms, FP64 state).
#include "launch_defs.cuh"
namespace laps {
template void launch_passB<float, double>(cudaStream_t, int, Bufs<float, double>, PassArgs, PassK<float, double>, const Store<float>::C*, const CUtensorMap*);
}  // namespace laps
