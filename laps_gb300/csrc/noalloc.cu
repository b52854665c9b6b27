// Forward 3-D transform of real FP64 fields that allocates no device memory.
//
// Some hosts cannot call cudaMalloc: a Fortran or C code whose device memory is handed out
// by its own pool or by a framework, a caller running where allocation is forbidden after
// start-up, or one that must not trigger the allocator's implicit synchronisation.  This
// entry point lets them run the engine's forward transform (the same kernels as
// laps_upload_state) on device buffers they already own.  The only extra device memory is
// the intermediate half spectrum of one field, kept in a fixed file-scope array that every
// GPU loading the library holds until the process exits.
#include <string>
#include "launch.cuh"

namespace laps {

// complex elements of the scratch half spectrum: room for one field of a 128^3 grid
constexpr long long NOALLOC_MAX_ELEMS = 1LL << 21;  // 32 MiB of double2

static __device__ __align__(256) double2 g_noalloc_scratch[NOALLOC_MAX_ELEMS];
static __device__ __align__(256) double2 g_noalloc_tw[3 * 512];  // x, y, z tables at 0, 512, 1024

// exp(-2 pi i j / n) for the three axes
__global__ void k_noalloc_twiddles(double2* tw, int nx, int ny, int nz) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int ns[3] = {nx, ny, nz};
  for (int a = 0; a < 3; a++) {
    if (j < ns[a]) {
      double s, c;
      sincospi(2.0 * (double)j / (double)ns[a], &s, &c);
      tw[a * 512 + j] = make_double2(c, -s);
    }
  }
}

// padded rows (pitch kxp) -> the reference's (nx/2+1, ny, nz) layout
__global__ void k_noalloc_unpad(const double2* __restrict__ in, double2* __restrict__ out, int nh, int kxp, long long rows) {
  long long tot = rows * nh;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot; i += (long long)gridDim.x * blockDim.x)
    out[i] = in[(i / nh) * kxp + i % nh];
}

static bool pow2_in(int n, int lo, int hi) { return n >= lo && n <= hi && (n & (n - 1)) == 0; }

}  // namespace laps

// error text for callers that have no context (shared with laps_last_error(NULL))
extern "C" const char* laps_last_error(struct laps_ctx*);
void laps_set_create_error(const std::string& m);

extern "C" int laps_transform_uu_real_to_fourier_noalloc(const double* uu, double* uf, int nx, int ny, int nz, int nfields,
                                                         void* stream) {
  using namespace laps;
  if (!uu || !uf || nfields < 1) {
    laps_set_create_error("noalloc transform: null buffer or nfields < 1");
    return LAPS_EINVAL;
  }
  if (!pow2_in(nx, 16, 512) || !pow2_in(ny, 8, 512) || !pow2_in(nz, 8, 512)) {
    laps_set_create_error("noalloc transform: nx must be a power of two in [16,512], ny and nz in [8,512]");
    return LAPS_EINVAL;
  }
  const int nh = nx / 2 + 1, kxp = (nh + 7) / 8 * 8;
  const long long need = (long long)kxp * ny * nz;
  if (need > NOALLOC_MAX_ELEMS) {
    laps_set_create_error("noalloc transform: grid too large for the fixed scratch (needs " + std::to_string(need) +
                          " complex elements, at most " + std::to_string(NOALLOC_MAX_ELEMS) + ")");
    return LAPS_EINVAL;
  }
  cudaStream_t s = (cudaStream_t)stream;
  try {
    // The arrays' device addresses are looked up on every call, with the caller's device and
    // context current: a cached address would go stale when the host resets the device
    // (cudaDeviceReset reloads the module at new addresses) or switches contexts, and the
    // lookup allocates nothing.  The first lookup in a context loads the module there.
    void* p = nullptr;
    LAPS_CK(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    double2* scr = (double2*)p;
    LAPS_CK(cudaGetSymbolAddress(&p, g_noalloc_tw));
    double2* tw = (double2*)p;
    k_noalloc_twiddles<<<2, 256, 0, s>>>(tw, nx, ny, nz);
    LAPS_CK(cudaGetLastError());
    const long long rows = (long long)ny * nz;
    for (int f = 0; f < nfields; f++) {
      const double* in = uu + (long long)f * nx * rows;
      double2* out = reinterpret_cast<double2*>(uf) + (long long)f * nh * rows;
      // x: r2c / nx into the padded scratch rows (every column later read is written here,
      // so nothing in the scratch has to start at zero)
      launch_rows_r2c<double>(s, nx, in, scr, rows, kxp, tw);
      // y and z: in place on the scratch, each divided by its length
      launch_col_plain<double>(s, scr, scr, 0, 1, ny, -1, kxp, ny * kxp, nh, nz, -ilog2(ny), tw + 512);
      launch_col_plain<double>(s, scr, scr, 0, 1, nz, -1, ny * kxp, kxp, nh, ny, -ilog2(nz), tw + 1024);
      k_noalloc_unpad<<<512, 256, 0, s>>>(scr, out, nh, kxp, rows);
      LAPS_CK(cudaGetLastError());
    }
  } catch (const Error& e) {
    laps_set_create_error("noalloc transform: " + e.msg);
    return e.code;
  }
  return LAPS_OK;
}
