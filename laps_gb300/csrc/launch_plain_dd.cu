// Plain transform launchers (dd).
#include "launch_defs.cuh"
namespace laps {
template void launch_col_plain<dd>(cudaStream_t, const Store<dd>::C*, Store<dd>::C*, long long, int, int, int, int, int, int, int, int, const Store<dd>::C*);
template void launch_rows_r2c<dd>(cudaStream_t, int, const Store<dd>::R*, Store<dd>::C*, long long, int, const Store<dd>::C*);
template void launch_rows_c2r<dd>(cudaStream_t, int, const Store<dd>::C*, Store<dd>::R*, long long, int, const Store<dd>::C*);
}  // namespace laps
