// Pass C launcher (float transforms, dd state, incompressible, CFL 1).
#include "launch_defs.cuh"
namespace laps {
template void launch_passC_v<float, dd, 1, 1>(cudaStream_t, int, Bufs<float, dd>, PassArgs, PassK<float, dd>, const Store<float>::C*);
}  // namespace laps
