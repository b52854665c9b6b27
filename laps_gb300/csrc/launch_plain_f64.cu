// Plain transform launchers (double).
#include "launch_defs.cuh"
namespace laps {
template void launch_col_plain<double>(cudaStream_t, const Store<double>::C*, Store<double>::C*, long long, int, int, int, int, int, int, int, int, const Store<double>::C*);
template void launch_rows_r2c<double>(cudaStream_t, int, const Store<double>::R*, Store<double>::C*, long long, int, const Store<double>::C*);
template void launch_rows_c2r<double>(cudaStream_t, int, const Store<double>::C*, Store<double>::R*, long long, int, const Store<double>::C*);
}  // namespace laps
