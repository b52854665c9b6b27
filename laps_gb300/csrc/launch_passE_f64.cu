// Pass E launcher (double transforms, double state).
#include "launch_defs.cuh"
namespace laps {
template void launch_passE<double, double>(cudaStream_t, int, Bufs<double, double>, PassArgs, PassK<double, double>, const Store<double>::C*, const CUtensorMap*);
template void launch_mass_rk<double, double>(cudaStream_t, Bufs<double, double>, PassArgs, PassK<double, double>);
}  // namespace laps
