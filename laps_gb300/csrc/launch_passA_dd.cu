// Pass A launcher (dd transforms, dd state).
#include "launch_defs.cuh"
namespace laps {
template void launch_passA<dd, dd>(cudaStream_t, int, Bufs<dd, dd>, PassArgs, PassK<dd, dd>, const Store<dd>::C*, const CUtensorMap*);
}  // namespace laps
