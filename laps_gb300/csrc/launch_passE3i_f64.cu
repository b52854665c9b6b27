// Incompressible pass E launcher (double).
#include "launch_defs.cuh"
namespace laps {
template void launch_passE3i<double>(cudaStream_t, int, Bufs<double>, PassArgs, PT<double>, KTab<double>, const Store<double>::C*);
}  // namespace laps
