// Pass E launcher (float transforms, dd state).
#include "launch_defs.cuh"
namespace laps {
template void launch_passE<float, dd>(cudaStream_t, int, Bufs<float, dd>, PassArgs, PassK<float, dd>, const Store<float>::C*, const CUtensorMap*);
template void launch_mass_rk<float, dd>(cudaStream_t, Bufs<float, dd>, PassArgs, PassK<float, dd>);
}  // namespace laps
