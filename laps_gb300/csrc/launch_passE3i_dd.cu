// Incompressible pass E launcher (dd).
#include "launch_defs.cuh"
namespace laps {
template void launch_passE3i<dd>(cudaStream_t, int, Bufs<dd>, PassArgs, PT<dd>, KTab<dd>, const Store<dd>::C*);
}  // namespace laps
