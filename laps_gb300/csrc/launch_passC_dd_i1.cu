// Pass C launcher (dd, incompressible, CFL 1).
#include "launch_defs.cuh"
namespace laps {
template void launch_passC_v<dd, 1, 1>(cudaStream_t, int, Bufs<dd>, PassArgs, PT<dd>, const Store<dd>::C*);
}  // namespace laps
