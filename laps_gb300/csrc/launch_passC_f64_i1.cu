// Pass C launcher (double transforms, double state, incompressible, CFL 1).
#include "launch_defs.cuh"
namespace laps {
template void launch_passC_v<double, double, 1, 1>(cudaStream_t, int, Bufs<double, double>, PassArgs, PassK<double, double>, const Store<double>::C*);
}  // namespace laps
