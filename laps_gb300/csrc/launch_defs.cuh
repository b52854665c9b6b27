// Definitions of the kernel launchers declared in launch.cuh.
#pragma once
#include "launch.cuh"

namespace laps {

template <class T>
void launch_col_plain(cudaStream_t stream, const typename Store<T>::C* in, typename Store<T>::C* out, long long fs, int nf, int N,
                      int dir, int jstride, int ostride, int ncol, int nouter, int sexp, const typename Store<T>::C* tw) {
#define LAPS_CASE(NN)                                                                                                   \
  case NN: {                                                                                                            \
    using CL = Col<T, NN>;                                                                                              \
    dim3 grid((ncol + TX - 1) / TX, (nouter + CL::NTILE - 1) / CL::NTILE, nf);                                          \
    if (dir < 0) {                                                                                                      \
      set_smem(k_col_plain<T, NN, -1>, CL::SMEM);                                                                       \
      k_col_plain<T, NN, -1><<<grid, CL::THREADS, CL::SMEM, stream>>>(in, out, fs, jstride, ostride, ncol, nouter, sexp, tw); \
    } else {                                                                                                            \
      set_smem(k_col_plain<T, NN, 1>, CL::SMEM);                                                                        \
      k_col_plain<T, NN, 1><<<grid, CL::THREADS, CL::SMEM, stream>>>(in, out, fs, jstride, ostride, ncol, nouter, sexp, tw); \
    }                                                                                                                   \
    break;                                                                                                              \
  }
  switch (N) { LAPS_COL_SIZES(LAPS_CASE) default: throw Error{LAPS_EINVAL, "unsupported column length"}; }
#undef LAPS_CASE
  LAPS_CK(cudaGetLastError());
}

template <class T>
void launch_rows_r2c(cudaStream_t stream, int nx, const typename Store<T>::R* in, typename Store<T>::C* out, long long nrows, int kxp,
                     const typename Store<T>::C* twx) {
#define LAPS_CASE(NN)                                                                                                   \
  case NN: {                                                                                                            \
    int sm = RowP<NN>::LB * RowP<NN>::LC * (int)sizeof(typename Store<T>::C);                                                   \
    set_smem(k_row_r2c<T, NN>, sm);                                                                                     \
    k_row_r2c<T, NN><<<(unsigned)((nrows + RowP<NN>::LB - 1) / RowP<NN>::LB), 128, sm, stream>>>(in, out, nrows, kxp, -ilog2(NN), twx); \
    break;                                                                                                              \
  }
  switch (nx) { LAPS_ROW_SIZES(LAPS_CASE) default: throw Error{LAPS_EINVAL, "unsupported nx"}; }
#undef LAPS_CASE
  LAPS_CK(cudaGetLastError());
}

template <class T>
void launch_rows_c2r(cudaStream_t stream, int nx, const typename Store<T>::C* in, typename Store<T>::R* out, long long nrows, int kxp,
                     const typename Store<T>::C* twx) {
#define LAPS_CASE(NN)                                                                                                   \
  case NN: {                                                                                                            \
    int sm = RowP<NN>::LB * RowP<NN>::LC * (int)sizeof(typename Store<T>::C);                                                   \
    set_smem(k_row_c2r<T, NN>, sm);                                                                                     \
    k_row_c2r<T, NN><<<(unsigned)((nrows + RowP<NN>::LB - 1) / RowP<NN>::LB), 128, sm, stream>>>(in, out, nrows, kxp, twx); \
    break;                                                                                                              \
  }
  switch (nx) { LAPS_ROW_SIZES(LAPS_CASE) default: throw Error{LAPS_EINVAL, "unsupported nx"}; }
#undef LAPS_CASE
  LAPS_CK(cudaGetLastError());
}

#define LAPS_COL_PASS(NAME, KERNEL, NOUTER)                                                                              \
  template <class T, class TS>                                                                                          \
  void NAME(cudaStream_t stream, int N, Bufs<T, TS> B, PassArgs a, PassK<T, TS> kk, const typename Store<T>::C* tw,   \
            const CUtensorMap* tm) {                                                                                   \
    switch (N) { LAPS_COL_SIZES(LAPS_CASE) default: throw Error{LAPS_EINVAL, "unsupported line length"}; }               \
    LAPS_CK(cudaGetLastError());                                                                                        \
  }
#define LAPS_CASE(NN)                                                                                                   \
  case NN: {                                                                                                            \
    using CL = Col<T, NN>;                                                                                              \
    /* the state tiles, which the transform tiles overwrite once every thread has read its elements */             \
    const int sm = CL::NTILE * NN * TX * (int)sizeof(typename Store<TS>::C);                                            \
    set_smem(k_passA<T, TS, NN>, sm);                                                                                   \
    dim3 grid((a.g.kx_keep + TX - 1) / TX, (a.g.nky() + CL::NTILE - 1) / CL::NTILE,                                     \
              a.P.variant == LAPS_VARIANT_3DI ? 12 : (a.hall ? 10 : 8));                                                \
    k_passA<T, TS, NN><<<grid, CL::THREADS, sm, stream>>>(B, a, kk, tw, *tm);                                           \
    break;                                                                                                              \
  }
LAPS_COL_PASS(launch_passA, k_passA, nky)
#undef LAPS_CASE
#define LAPS_CASE(NN)                                                                                                   \
  case NN: {                                                                                                            \
    using CL = Col<T, NN>;                                                                                              \
    /* 2-D: one buffer per tile (the state is read by the threads) - tiles are laid out with */                      \
    /* two buffers each, so only a single-tile block may drop the second; 3-D: the two inputs  */                      \
    const int smB = ((a.P.two_d || PassBOneBuf<T, NN>::V) && CL::NTILE == 1) ? CL::SMEM : 2 * CL::SMEM;                 \
    if (!a.P.two_d && col_one_buffer<T, NN>()) throw Error{LAPS_EINVAL, "column tiles exceed shared memory"};             \
    dim3 grid((a.g.kx_keep + TX - 1) / TX, (a.g.nz + CL::NTILE - 1) / CL::NTILE,                                        \
              a.P.variant == LAPS_VARIANT_3DI ? 19 : (a.hall ? 11 : 8));                                                \
    /* FP32 lines up to 256 points: persistent blocks with two buffer sets (>= 3 blocks per SM) */                   \
    if ((a.sched & LAPS_SCHED_PERSISTENT_B) && !a.P.two_d && sizeof(typename Store<T>::C) == 8 && 4 * CL::SMEM <= 72 * 1024) { \
      const int smP = 4 * CL::SMEM;                                                                                     \
      set_smem(k_passB_pipe<T, TS, NN>, smP);                                                                           \
      const int nitems = grid.x * grid.y * grid.z;                                                                      \
      const int pb = persistent_blocks(k_passB_pipe<T, TS, NN>, CL::THREADS, smP);                                      \
      k_passB_pipe<T, TS, NN><<<nitems < pb ? nitems : pb, CL::THREADS, smP, stream>>>(B, a, kk, tw, *tm, nitems,      \
                                                                                       grid.x, grid.y);                 \
      break;                                                                                                            \
    }                                                                                                                   \
    set_smem(k_passB<T, TS, NN>, smB);                                                                                  \
    k_passB<T, TS, NN><<<grid, CL::THREADS, smB, stream>>>(B, a, kk, tw, *tm);                                          \
    break;                                                                                                              \
  }
LAPS_COL_PASS(launch_passB, k_passB, nz)
#undef LAPS_CASE
#define LAPS_CASE(NN)                                                                                                   \
  case NN: {                                                                                                            \
    using CL = Col<T, NN>;                                                                                              \
    const int smD = col_one_buffer<T, NN>() ? CL::SMEM : 2 * CL::SMEM;                                                  \
    set_smem(k_passD<T, TS, NN>, smD);                                                                                  \
    dim3 grid((a.g.kx_keep + TX - 1) / TX, (a.g.nz + CL::NTILE - 1) / CL::NTILE, a.P.variant == LAPS_VARIANT_3DI ? 5 : (a.mass_from_state ? 6 : 8)); \
    k_passD<T, TS, NN><<<grid, CL::THREADS, smD, stream>>>(B, a, kk, tw, *tm);                                          \
    break;                                                                                                              \
  }
LAPS_COL_PASS(launch_passD, k_passD, nz)
#undef LAPS_CASE
#define LAPS_CASE(NN)                                                                                                   \
  case NN: {                                                                                                            \
    using CL = Col<T, NN>;                                                                                              \
    set_smem(k_passE<T, TS, NN>, 2 * CL::SMEM);                                                                         \
    dim3 grid((a.g.kx_keep + TX - 1) / TX, (a.g.nky() + CL::NTILE - 1) / CL::NTILE, 8);                                  \
    PassArgs a0 = a;                                                                                                    \
    a0.e_first = 0;                                                                                                     \
    if (a.mass_from_state) { /* continuity from the momentum first, then variables 1..7 */                             \
      if (!a.mass_done) launch_mass_rk<T, TS>(stream, B, a, kk);                                                        \
      a0.e_first = 1;                                                                                                   \
      grid.z = 7;                                                                                                       \
    }                                                                                                                   \
    if constexpr (NN == 1) { /* 2-D: the elementwise form */                                                          \
      const long long tot = (long long)a.g.kx_keep * a.g.nky();                                                        \
      const long long nb = (tot + 255) / 256;                                                                           \
      k_passE2d<T, TS><<<dim3((unsigned)(nb < 1216 ? nb : 1216), grid.z), 256, 0, stream>>>(B, a0, kk,                   \
                                                                                               FastDiv(a.g.kx_keep));  \
      break;                                                                                                            \
    }                                                                                                                   \
    k_passE<T, TS, NN><<<grid, CL::THREADS, 2 * CL::SMEM, stream>>>(B, a0, kk, tw, tm[0], tm[1], tm[2]);                                     \
    break;                                                                                                              \
  }
LAPS_COL_PASS(launch_passE, k_passE, nky)
#undef LAPS_CASE
#define LAPS_CASE(NN)                                                                                                   \
  case NN: {                                                                                                            \
    using CL = Col<T, NN>;                                                                                              \
    set_smem(k_passE3i<T, TS, NN>, 3 * CL::SMEM);                                                                           \
    dim3 grid((a.g.kx_keep + TX - 1) / TX, (a.g.nky() + CL::NTILE - 1) / CL::NTILE, 4);                                  \
    k_passE3i<T, TS, NN><<<grid, CL::THREADS, 3 * CL::SMEM, stream>>>(B, a, kk, tw);                                     \
    break;                                                                                                              \
  }
LAPS_COL_PASS(launch_passE3i, k_passE3i, nky)
#undef LAPS_CASE
#undef LAPS_COL_PASS

// pass C for one (physics, CFL) combination; each combination is instantiated in its own
// translation unit (launch_passC_<type>_<c|i><0|1>.cu)
template <class T, class TS, int INCOMP, int CFL>
void launch_passC_v(cudaStream_t stream, int N, Bufs<T, TS> B, PassArgs a, PassK<T, TS> kk, const typename Store<T>::C* tw) {
#define LAPS_CASE(NN)                                                                                                   \
  case NN: {                                                                                                            \
    using CF = PassCCfg<NN, (int)sizeof(typename Store<T>::C)>;                                                         \
    unsigned nb = (unsigned)((long long)a.g.ny * a.g.nz / CF::ROWS);                                                    \
    set_smem(k_passC<T, TS, NN, CFL, INCOMP>, CF::SMEM);                                                                \
    k_passC<T, TS, NN, CFL, INCOMP><<<nb, CF::THREADS, CF::SMEM, stream>>>(B, a, kk, tw);                               \
    break;                                                                                                              \
  }
  switch (N) { LAPS_ROW_SIZES(LAPS_CASE) default: throw Error{LAPS_EINVAL, "unsupported nx"}; }
#undef LAPS_CASE
  LAPS_CK(cudaGetLastError());
}

// the continuity update alone (forked beside pass D by the step)
template <class T, class TS>
void launch_mass_rk(cudaStream_t stream, Bufs<T, TS> B, PassArgs a, PassK<T, TS> kk) {
  const long long tot = (long long)a.g.kx_keep * a.g.nky() * a.g.nkz();
  const FastDiv dkx(a.g.kx_keep), dky(a.g.nky());
  if (tot < (1ll << 31)) k_mass_rk<T, TS, unsigned><<<mass_rk_blocks(a.g), 256, 0, stream>>>(B, a, kk, dkx, dky);
  else k_mass_rk<T, TS, long long><<<mass_rk_blocks(a.g), 256, 0, stream>>>(B, a, kk, dkx, dky);
  LAPS_CK(cudaGetLastError());
}

}  // namespace laps
