// Pass E launcher (float transforms, FP64 state).
#include "launch_defs.cuh"
namespace laps {
template void launch_passE<float, double>(cudaStream_t, int, Bufs<float, double>, PassArgs, PassK<float, double>, const Store<float>::C*, const CUtensorMap*);
template void launch_mass_rk<float, double>(cudaStream_t, Bufs<float, double>, PassArgs, PassK<float, double>);
}  // namespace laps
