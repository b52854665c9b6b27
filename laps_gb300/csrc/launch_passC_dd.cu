// Pass C launcher (dd).
#include "launch_defs.cuh"
namespace laps {
template void launch_passC<dd>(cudaStream_t, int, Bufs<dd>, PassArgs, PT<dd>, const Store<dd>::C*);
}  // namespace laps
