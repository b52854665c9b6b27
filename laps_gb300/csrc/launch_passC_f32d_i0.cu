// Pass C launcher (float transforms, FP64 state, incompressible, CFL 0).
#include "launch_defs.cuh"
namespace laps {
template void launch_passC_v<float, double, 1, 0>(cudaStream_t, int, Bufs<float, double>, PassArgs, PassK<float, double>, const Store<float>::C*);
}  // namespace laps
