// Pass C launcher (dd transforms, dd state, compressible, CFL 0).
#include "launch_defs.cuh"
namespace laps {
template void launch_passC_v<dd, dd, 0, 0>(cudaStream_t, int, Bufs<dd, dd>, PassArgs, PassK<dd, dd>, const Store<dd>::C*);
}  // namespace laps
