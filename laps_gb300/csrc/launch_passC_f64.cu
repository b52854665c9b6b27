// Pass C launcher (double).
#include "launch_defs.cuh"
namespace laps {
template void launch_passC<double>(cudaStream_t, int, Bufs<double>, PassArgs, PT<double>, const Store<double>::C*);
}  // namespace laps
