// Pass C launcher (float transforms, dd state, compressible, CFL 0).
#include "launch_defs.cuh"
namespace laps {
template void launch_passC_v<float, dd, 0, 0>(cudaStream_t, int, Bufs<float, dd>, PassArgs, PassK<float, dd>, const Store<float>::C*);
}  // namespace laps
