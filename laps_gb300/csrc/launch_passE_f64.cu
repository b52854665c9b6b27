// Pass E launcher (double).
#include "launch_defs.cuh"
namespace laps {
template void launch_passE<double>(cudaStream_t, int, Bufs<double>, PassArgs, PT<double>, KTab<double>, const Store<double>::C*);
}  // namespace laps
