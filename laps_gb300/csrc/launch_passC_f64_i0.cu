// Pass C launcher (double, incompressible, CFL 0).
#include "launch_defs.cuh"
namespace laps {
template void launch_passC_v<double, 1, 0>(cudaStream_t, int, Bufs<double>, PassArgs, PT<double>, const Store<double>::C*);
}  // namespace laps
