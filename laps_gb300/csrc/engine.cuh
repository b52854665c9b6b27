// Device-side definitions shared by every kernel of the engine: grid geometry, the
// per-step scalars that live in device memory (so a captured step needs no host input),
// wave-number tables and the pointwise physics of the 3-D compressible equations.
#pragma once
#include "fft.cuh"
#include "laps_gpu.h"

namespace laps {

constexpr int TX = 8;  // columns per tile: 8 x 16 B = one 128-byte row

// ------------------------------------------------------------------------------ geometry
// Spectral / intermediate arrays: field-major, then z, y, and kx fastest with a row pitch
// kxp = round_up(nx/2+1, 8), i.e. the reference's uu_fourier(kx,ky,kz,ivar) order
// (src_compressible/mhdinit.f90:155-169) with padded rows.  Real arrays: (x, y, z, field)
// exactly as the reference's uu(ix,iy,iz,ivar).
// q = n / d for 0 <= n < 2^31 by one multiply-high, an add and a shift (Granlund & Montgomery,
// "Division by invariant integers using multiplication", PLDI 1994): with l = ceil(log2 d) and
// m = floor(2^32 (2^l - d) / d) + 1, n / d = (mulhi(n, m) + n) >> l; the sum stays below 2^32
// for n < 2^31.  The magic numbers come from the host; on this GPU a runtime integer division
// costs conversion instructions, which run on the slow FP64 pipe.
struct FastDiv {
  unsigned d, m, l;
  FastDiv() = default;
  explicit FastDiv(unsigned div) : d(div), m(0), l(0) {
    while ((1ull << l) < div) l++;
    m = (unsigned)((((1ull << 32) * ((1ull << l) - div)) / div) + 1);
  }
  __host__ __device__ __forceinline__ unsigned div(unsigned n) const {
#ifdef __CUDA_ARCH__
    return (__umulhi(n, m) + n) >> l;
#else
    return (unsigned)((((unsigned long long)n * m >> 32) + n) >> l);
#endif
  }
};

struct Geo {
  int nx, ny, nz, nh;     // nh = nx/2 + 1
  int kxp;                // spectral row pitch
  long long fsc;          // complex field stride = nz*ny*kxp
  long long fsr;          // real field stride = nz*ny*nx
  // kept (non-zero) spectral ranges: kx < kx_keep, ky in [0,ky_lo) U [ky_hi,ny), same for kz
  int kx_keep, ky_lo, ky_hi, kz_lo, kz_hi;
  __host__ __device__ int nky() const { return ky_lo + (ny - ky_hi); }
  __host__ __device__ int nkz() const { return kz_lo + (nz - kz_hi); }
  __host__ __device__ int ky_of(int r) const { return r < ky_lo ? r : ky_hi + (r - ky_lo); }
  __host__ __device__ int kz_of(int r) const { return r < kz_lo ? r : kz_hi + (r - kz_lo); }
  __host__ __device__ bool ky_in(int ky) const { return ky < ky_lo || ky >= ky_hi; }
  __host__ __device__ bool kz_in(int kz) const { return kz < kz_lo || kz >= kz_hi; }
};

// Tile copies of a line whose kept rows are [0, lo) U [hi, n): boxes of `box` rows at 0, box,
// 2 box, ... below lo_end and at n - box, n - 2 box, ... down to hi_start, so that the unkept
// middle is not fetched.  `box` is a multiple of `gran` rows (n a power of two), so that every
// copy lands on a 128-byte boundary of shared memory (gran = 128 / tile row bytes).  When the
// two runs of boxes would overlap (little or no dealiasing) the whole line is copied in boxes
// of min(n, 256) rows from 0 and the high run is empty.
struct KeptCopies {
  int box, lo_end, hi_start;  // low run covers [0, lo_end), high run [hi_start, n)
  __host__ __device__ KeptCopies(int lo, int hi, int n, int gran) {
    const int nh = n - hi, full = n < 256 ? n : 256;
    int kb = lo > nh ? lo : nh;
    kb = kb < 1 ? 1 : kb;
    const int parts = (kb + 255) / 256;  // boxes of at most 256 rows, as even as they come
    kb = (kb + parts - 1) / parts;
    kb = (kb + gran - 1) / gran * gran;
    const bool split = kb <= full && (lo + kb - 1) / kb * kb + (nh + kb - 1) / kb * kb <= n;
    box = split ? kb : full;
    lo_end = split ? lo : n;
    hi_start = split ? hi : n;
  }
  // number of box copies per line
  __host__ __device__ int count(int n) const { return (lo_end + box - 1) / box + (n - hi_start + box - 1) / box; }
  // start row of copy i (i < count(n))
  __host__ __device__ int start(int i, int n) const {
    const int nl = (lo_end + box - 1) / box;
    return i < nl ? i * box : n - (i - nl + 1) * box;
  }
};
// rows of TX complex elements of `bytes` each that make 128 bytes
__host__ __device__ constexpr int tile_gran(int bytes) { return 128 / (TX * bytes) > 1 ? 128 / (TX * bytes) : 1; }

// ------------------------------------------------------------------------------ step state
// Written only by device kernels during a step; read by every pass kernel.
struct StepState {
  double time, dt, radius;
  double cc[3], ddc[3], ts[3];     // RK3 coefficients of rktmod.f90:17-27 times dt
  double inv_tau;                  // 1 / tau_exp (0 when the expanding box is off)
  double r_ratio;                  // radius0 / radius
  unsigned long long cfl_bits;     // running min of the CFL time step (bits of a double)
  double rho0;                     // 3-D incompressible background density (update_rho_p)
  long long istep;                 // steps taken (2-D vardt cadence)
  int status;                      // LAPS_STATUS_* bits
  int halt;                        // skip the rest of the step (dt floor)
  int ksq_plain;                   // k^2 still the grid_initialize sum (no R factor)
  unsigned int cfl32_bits;         // running min of the FP32 screen of the CFL step (bits of a float)
  // the nearest floats of cc, ddc, ts, inv_tau and r_ratio for the FP32-increment updates,
  // written with them (step_state_f32): a conversion from binary64 (and a binary64 division)
  // issues at the FP64 pipe's rate on this GPU, too slow to repeat in every thread
  float f_cc[3], f_ddc[3], f_ts[3], f_inv_tau, f_r_ratio;
  double inv_rho0;  // 1 / rho0, with its nearest float
  float f_inv_rho0;
  double R0;        // radius0 (constant), and radius / radius0 with its nearest float (CFL)
  double rfac;
  float f_rfac;
};
__host__ __device__ inline void step_state_f32(StepState& s) {
  for (int i = 0; i < 3; i++) {
    s.f_cc[i] = (float)s.cc[i];
    s.f_ddc[i] = (float)s.ddc[i];
    s.f_ts[i] = (float)s.ts[i];
  }
  s.f_inv_tau = (float)s.inv_tau;
  s.f_r_ratio = (float)s.r_ratio;
  s.inv_rho0 = 1.0 / s.rho0;
  s.f_inv_rho0 = (float)s.inv_rho0;
  s.rfac = s.radius / s.R0;
  s.f_rfac = (float)s.rfac;
}

// wave-number tables (element type T), rebuilt by a small kernel whenever R changes
template <class T> struct KTab {
  const T* wx;   // kx (nh)
  const T* kxd;  // kx derivative factor: kx, or kx * R0 / R when z is radial (2-D)
  const T* wy;   // ky (ny) unscaled
  const T* kyd;  // ky * R0 / R   (derivative factor)
  const T* kzd;  // kz * R0 / R
  const T* kx2;  // terms of k^2: kx^2, (ky R0/R)^2, (kz R0/R)^2 (plain squares before the first R update)
  const T* ky2;
  const T* kz2;
  const T* fx;   // dealias option 2 filters (or null)
  const T* fy;
  const T* fz;
  const short* kxlim;  // dealias option 1: number of kept kx for each (kz, ky) row, or null
};

// scalar physics parameters, by value
struct Phys {
  double gamma, nu, eta, di, cfl, dx, dy, dz, mindx, R0, Ur;
  double cos_cor, sin_cor;
  int visc, visc_exp, resis, resis_exp, cons_bg, aeb, corot, hall, dealias;
  int variant;   // LAPS_VARIANT_*
  int two_d;     // nz == 1: kz = 0, no z term in the CFL
  int zrad;      // 2-D expanding box with z radial
  int limit_dt;  // 2-D if_limit_dt_increase
  int dstep;     // vardt cadence (steps)
  int ebm_mask;  // variables damped by the expansion (bit v)
};

// the same constants pre-converted to T on the host (a double -> float-float split per
// element would run on the FP64 pipe)
template <class T> struct PT {
  T gamma, gm1, cg, di, nu, eta, cosc, sinc, inv_mindx, half, two, one, zero, four, is2, dx, dy, dz;
  T eta_dx, eta_dy;  // explicit-resistivity CFL speeds (2-D)
  T ebm[8];          // expansion damping factor of each variable
};

// the constants in FP32 (the CFL screen)
template <class T> __device__ __forceinline__ PT<float> pt_float(const PT<T>& c) {
  PT<float> f;
  f.gamma = Cvt<float, T>::r(c.gamma); f.gm1 = Cvt<float, T>::r(c.gm1); f.cg = Cvt<float, T>::r(c.cg);
  f.di = Cvt<float, T>::r(c.di); f.nu = Cvt<float, T>::r(c.nu); f.eta = Cvt<float, T>::r(c.eta);
  f.cosc = Cvt<float, T>::r(c.cosc); f.sinc = Cvt<float, T>::r(c.sinc); f.inv_mindx = Cvt<float, T>::r(c.inv_mindx);
  f.half = 0.5f; f.two = 2.f; f.one = 1.f; f.zero = 0.f; f.four = 4.f; f.is2 = Cvt<float, T>::r(c.is2);
  f.dx = Cvt<float, T>::r(c.dx); f.dy = Cvt<float, T>::r(c.dy); f.dz = Cvt<float, T>::r(c.dz);
  f.eta_dx = Cvt<float, T>::r(c.eta_dx); f.eta_dy = Cvt<float, T>::r(c.eta_dy);
#pragma unroll
  for (int v = 0; v < 8; v++) f.ebm[v] = Cvt<float, T>::r(c.ebm[v]);
  return f;
}

// everything a pass needs in the compute type T and in the state type TS
template <class T, class TS> struct PassK {
  PT<T> pc;
  PT<TS> ps;
  KTab<T> K;
  KTab<TS> KS;
};

// effective derivative factors (i*ax, i*ay, i*az) at spectral index (ix, iy, iz):
// src_compressible/mhdrhs.f90:191-204 (corotation mixes kx and ky)
template <class T>
__device__ __forceinline__ void kfac(const KTab<T>& K, const Phys& P, const PT<T>& c, T rr, int ix, int iy, int iz, T& ax, T& ay, T& az) {
  az = K.kzd[iz];
  if (P.corot) {
    ax = K.wx[ix] * c.cosc + K.wy[iy] * c.sinc;
    ay = (K.wy[iy] * c.cosc - K.wx[ix] * c.sinc) * rr;
  } else {
    ax = K.kxd[ix];
    ay = K.kyd[iy];
  }
}

// k^2 at (ix, iy, iz): src_compressible/AEBmod.f90:87-125 and mhdinit.f90:117-123
template <class T>
__device__ __forceinline__ T ksq(const KTab<T>& K, const Phys& P, const PT<T>& q, T rr, int ix, int iy, int iz) {
  if (P.corot) {
    T c = q.cosc, s = q.sinc;
    T kx = K.wx[ix], ky = K.wy[iy];
    T r2 = rr * rr;
    T sr = s * rr, cr = c * rr;
    return kx * kx * (c * c + sr * sr) + ky * ky * (s * s + cr * cr) + kx * ky * q.two * c * s * (q.one - r2) + K.kz2[iz];
  }
  return (K.kx2[ix] + K.ky2[iy]) + K.kz2[iz];
}

}  // namespace laps
