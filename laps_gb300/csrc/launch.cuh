// Kernel launchers, one switch over the supported line lengths per pass.  Each launcher
// is explicitly instantiated per element type in its own translation unit (launch_*.cu)
// so that the float-float FFT code compiles in parallel.
#pragma once
#include <cuda.h>
#include <cudaTypedefs.h>
#include <string>
#include "passes.cuh"

namespace laps {

inline int ilog2(int n) { int l = 0; while ((1 << l) < n) l++; return l; }

struct Error {
  int code;
  std::string msg;
};

#define LAPS_CK(call)                                                                    \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess) throw Error{LAPS_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)}; \
  } while (0)

#define LAPS_COL_SIZES(X) X(1) X(8) X(16) X(32) X(64) X(128) X(256) X(512) X(1024)
#define LAPS_ROW_SIZES(X) X(16) X(32) X(64) X(128) X(256) X(512) X(1024)

// opt in to more than the default 48 KB per block; the default covers static and dynamic shared
// memory together, so requests close to it opt in too (kernels keep < 8 KB static)
// blocks of the continuity update: four per SM, or fewer when the kept modes are fewer
inline int mass_rk_blocks(const Geo& g) {
  const long long tot = (long long)g.kx_keep * g.nky() * g.nkz();
  const long long nb = (tot + 255) / 256;
  return (int)(nb < 4 * 152 ? (nb > 0 ? nb : 1) : 4 * 152);
}

// cuTensorMapEncodeTiled from the driver, looked up once through the runtime
inline PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    LAPS_CK(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q));
    if (q != cudaDriverEntryPointSuccess || !p) throw Error{LAPS_ECUDA, "cuTensorMapEncodeTiled is not available"};
    fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

template <class K> inline void set_smem(K kernel, int bytes) {
  if (bytes > 40 * 1024) LAPS_CK(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
}

// persistent kernels: as many blocks as are resident at once on the device (at least one per SM)
template <class K> inline int persistent_blocks(K kernel, int threads, int smem) {
  int per_sm = 0, dev = 0, nsm = 0;
  LAPS_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem));
  LAPS_CK(cudaGetDevice(&dev));
  LAPS_CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  return (per_sm > 0 ? per_sm : 1) * nsm;
}


template <class T>
void launch_col_plain(cudaStream_t stream, const typename Store<T>::C* in, typename Store<T>::C* out, long long fs, int nf, int N,
                      int dir, int jstride, int ostride, int ncol, int nouter, int sexp, const typename Store<T>::C* tw);
template <class T>
void launch_rows_r2c(cudaStream_t stream, int nx, const typename Store<T>::R* in, typename Store<T>::C* out, long long nrows, int kxp,
                     const typename Store<T>::C* twx);
template <class T>
void launch_rows_c2r(cudaStream_t stream, int nx, const typename Store<T>::C* in, typename Store<T>::R* out, long long nrows, int kxp,
                     const typename Store<T>::C* twx);
template <class T, class TS> void launch_passA(cudaStream_t stream, int N, Bufs<T, TS> B, PassArgs a, PassK<T, TS> kk, const typename Store<T>::C* tw,
                                             const CUtensorMap* tm);
template <class T, class TS> void launch_passB(cudaStream_t stream, int N, Bufs<T, TS> B, PassArgs a, PassK<T, TS> kk, const typename Store<T>::C* tw,
                                             const CUtensorMap* tm);
template <class T, class TS, int INCOMP, int CFL>
void launch_passC_v(cudaStream_t stream, int N, Bufs<T, TS> B, PassArgs a, PassK<T, TS> kk, const typename Store<T>::C* tw);
template <class T, class TS>
void launch_passC(cudaStream_t stream, int N, Bufs<T, TS> B, PassArgs a, PassK<T, TS> kk, const typename Store<T>::C* tw) {
  if (a.P.variant == LAPS_VARIANT_3DI) {
    if (a.cfl) launch_passC_v<T, TS, 1, 1>(stream, N, B, a, kk, tw);
    else launch_passC_v<T, TS, 1, 0>(stream, N, B, a, kk, tw);
  } else {
    if (a.cfl) launch_passC_v<T, TS, 0, 1>(stream, N, B, a, kk, tw);
    else launch_passC_v<T, TS, 0, 0>(stream, N, B, a, kk, tw);
  }
}
template <class T, class TS> void launch_passD(cudaStream_t stream, int N, Bufs<T, TS> B, PassArgs a, PassK<T, TS> kk, const typename Store<T>::C* tw,
                                             const CUtensorMap* tm);
template <class T, class TS> void launch_passE(cudaStream_t stream, int N, Bufs<T, TS> B, PassArgs a, PassK<T, TS> kk, const typename Store<T>::C* tw,
                                             const CUtensorMap* tm);
template <class T, class TS> void launch_mass_rk(cudaStream_t stream, Bufs<T, TS> B, PassArgs a, PassK<T, TS> kk);
template <class T, class TS> void launch_passE3i(cudaStream_t stream, int N, Bufs<T, TS> B, PassArgs a, PassK<T, TS> kk, const typename Store<T>::C* tw,
                                             const CUtensorMap* tm);

}  // namespace laps
