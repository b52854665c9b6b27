// Pass E launcher (dd transforms, dd state).
#include "launch_defs.cuh"
namespace laps {
template void launch_passE<dd, dd>(cudaStream_t, int, Bufs<dd, dd>, PassArgs, PassK<dd, dd>, const Store<dd>::C*, const CUtensorMap*);
template void launch_mass_rk<dd, dd>(cudaStream_t, Bufs<dd, dd>, PassArgs, PassK<dd, dd>);
}  // namespace laps
