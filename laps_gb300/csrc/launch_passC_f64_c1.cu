// Pass C launcher (double, compressible, CFL 1).
#include "launch_defs.cuh"
namespace laps {
template void launch_passC_v<double, 0, 1>(cudaStream_t, int, Bufs<double>, PassArgs, PT<double>, const Store<double>::C*);
}  // namespace laps
