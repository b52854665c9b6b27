// Pass A launcher (double).
#include "launch_defs.cuh"
namespace laps {
template void launch_passA<double>(cudaStream_t, int, Bufs<double>, PassArgs, PT<double>, KTab<double>, const Store<double>::C*);
}  // namespace laps
