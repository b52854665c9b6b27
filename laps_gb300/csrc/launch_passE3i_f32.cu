// Pass E3i launcher (float transforms, dd state).
#include "launch_defs.cuh"
namespace laps {
template void launch_passE3i<float, dd>(cudaStream_t, int, Bufs<float, dd>, PassArgs, PassK<float, dd>, const Store<float>::C*, const CUtensorMap*);
}  // namespace laps
