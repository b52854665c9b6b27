// Kernels of the 3-D compressible step.  One RK stage is five passes over HBM:
//
//   A  inverse z-FFT of the state (+ the kz parts of J = ik x B)        U  -> W1
//   B  inverse y-FFT (+ the kx, ky parts of J)                          W1 -> W2
//   C  inverse x-FFT (c2r), fluxes, CFL, forward x-FFT (r2c)           W2 -> W1
//   D  forward y-FFT, kx/ky parts of -ik.F and curl E pre-combined     W1 -> W2
//   E  forward z-FFT, kz parts, expansion/diffusion, RK3, dealias      W2 -> U, R
//
// which replaces, per stage, calc_flux / transform_flux_real_to_fourier / calc_rhs / rkt /
// dealias / transform_uu_fourier_to_real / update_uu_prim_from_uu and, for the Hall term,
// calc_current_density_real (src_compressible/mhd.f90:303-325, mhdrhs.f90:21-362,
// rktmod.f90:34-62, dealiasing.f90:70-113, fftw.f90:73-222).  The reference's MPI pencil
// transposes (parallel.f90:218-324) have no counterpart: every pass reads its lines in
// 128-byte rows of TX = 8 adjacent columns from the fixed (kx, y, z) layout.
//
// With the spherical 2/3 mask (dealias_option 1) only |k_i| <= n_i/3 can be non-zero after
// the first stage, so the passes touch only that box (Geo::kx_keep, ky/kz ranges).
#pragma once
#include "engine.cuh"

namespace laps {

template <class T, int N> struct Col {
  using C = typename Store<T>::C;
  static constexpr int TPL = Plan<N>::TPL;
  static constexpr int NT = TX * TPL;  // threads per tile
  static constexpr int NTILE = NT >= 128 ? 1 : 128 / NT;
  static constexpr int THREADS = NT * NTILE;
  static constexpr int EPT = N / TPL;  // elements per thread
  static constexpr int SMEM = NTILE * N * TX * (int)sizeof(C);  // one buffer per tile
};

// Two column tiles of length N no longer fit one block's shared memory (1024-point columns of
// 16-byte elements: 2 x 128 KB): such passes keep one tile in shared memory and the other
// thread's-own elements in registers
template <class T, int N> __host__ __device__ constexpr bool col_one_buffer() { return 2 * Col<T, N>::SMEM > 220 * 1024; }

// T: the compute type of the transforms and products; TS: the storage type of the state
// and of the RK register (the same except in the FP32-transform mode, where TS is
// float-float)
template <class T, class TS = T> struct Bufs {
  typename Store<TS>::C* U;  // state spectrum, 8 fields
  typename Store<T>::C* R;   // fnl_rk, 8 fields (the right-hand side, in the transforms' type)
  typename Store<T>::C* W1;  // work, up to 19 fields
  typename Store<T>::C* W2;  // work, up to 19 fields
};

// --------------------------------------------------------------------------- plain transforms
// FFT along a column direction (y or z) of nf fields.  Element (f, outer, j, col) at
// f*fs + outer*ostride + j*jstride + col.  Forward results are multiplied by `scale`.
template <class T, int N, int DIR>
__global__ void __launch_bounds__(Col<T, N>::THREADS)
    k_col_plain(const typename Store<T>::C* __restrict__ in, typename Store<T>::C* __restrict__ out, long long fs,
                int jstride, int ostride, int ncol, int nouter, int scale_exp, const typename Store<T>::C* __restrict__ tw) {
  using CL = Col<T, N>;
  using C = typename Store<T>::C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* sm = reinterpret_cast<C*>(smem_raw);
  int tl = threadIdx.x / CL::NT, tid = threadIdx.x % CL::NT;
  int c = tid % TX, t = tid / TX;
  int col = blockIdx.x * TX + c;
  int outer = blockIdx.y * CL::NTILE + tl;
  long long base = (long long)blockIdx.z * fs + (long long)outer * ostride + col;
  C* s = sm + tl * N * TX;
  bool ok = col < ncol && outer < nouter;
#pragma unroll
  for (int m = 0; m < CL::EPT; m++) {
    int j = t + m * CL::TPL;
    cx<T> v = ok ? Store<T>::ldc(in + base + (long long)j * jstride) : cx_zero<T>();  // in may equal out
    Store<T>::stc(s + j * TX + c, v);
  }
  __syncthreads();
  fft_lines<T, N, DIR, TX, 1>(s, c, t, true, tw, 1);
  if (!ok) return;
#pragma unroll 4
  for (int m = 0; m < CL::EPT; m++) {
    int j = t + m * CL::TPL;
    cx<T> v = Store<T>::ldc(s + j * TX + c);
    if (scale_exp) v = {Real<T>::mul_pow2(v.re, scale_exp), Real<T>::mul_pow2(v.im, scale_exp)};
    Store<T>::stc(out + base + (long long)j * jstride, v);
  }
}

// Row helpers: a real row of NX values viewed as NX/2 complex (x[2m] + i x[2m+1]), stored
// in shared memory with one padding element after every 16 complex (sm_idx<1>).
template <int NX> struct RowP {
  static constexpr int H = NX / 2;
  static constexpr int TPL = Plan<H>::TPL;
  static constexpr int LB = 128 / TPL >= 1 ? 128 / TPL : 1;  // lines per batch of 128 threads
  static constexpr int LC = RowLen<H>::V;                    // padded line length (complex)
};
// real x of a padded row line, in Store<T>::R units
__device__ __forceinline__ int row_real_idx(int x) { return 2 * sm_idx<1>(x >> 1) + (x & 1); }

// c2r pre-processing of one line: Z[k] = (X[k] + conj X[h-k]) + i conj(W^k) (X[k] - conj X[h-k])
// for the pair (k, h-k); X read from global through `ldx`, imaginary parts of X[0], X[h] ignored.
template <class T, int H, class LDX>
__device__ __forceinline__ void c2r_pre(typename Store<T>::C* z, int t, LDX ldx, const typename Store<T>::C* __restrict__ twx) {
  constexpr int TPL = Plan<H>::TPL;
  auto pair = [&](int k, cx<T> a, cx<T> b) {
    const int k2 = H - k;
    if (k == 0) { a.im = Real<T>::cst(0.0); b.im = Real<T>::cst(0.0); }
    cx<T> wa = conj(Store<T>::ldg(twx + k));
    cx<T> za = (a + conj(b)) + times_i(wa * (a - conj(b)));
    if (k == 0) {
      Store<T>::stc(z, za);
    } else {
      cx<T> wb = conj(Store<T>::ldg(twx + k2));
      cx<T> zb = (b + conj(a)) + times_i(wb * (b - conj(a)));
      Store<T>::stc(z + sm_idx<1>(k), za);
      if (k2 != k) Store<T>::stc(z + sm_idx<1>(k2), zb);
    }
  };
  if constexpr (sizeof(typename Store<T>::C) == 8) {
    // FP32 lines: every load of the line's pairs first, then the arithmetic
    constexpr int NIT = (H / 2 + TPL) / TPL;  // pairs per thread
    cx<T> xa[NIT], xb[NIT];
#pragma unroll
    for (int i = 0; i < NIT; i++) {
      const int k = t + i * TPL;
      if (k <= H / 2) {
        xa[i] = ldx(k);
        xb[i] = ldx(H - k);
      }
    }
#pragma unroll
    for (int i = 0; i < NIT; i++) {
      const int k = t + i * TPL;
      if (k <= H / 2) pair(k, xa[i], xb[i]);
    }
  } else {  // wider types would not keep the pairs in registers
    for (int k = t; k <= H / 2; k += TPL) pair(k, ldx(k), ldx(H - k));
  }
}

// Two real rows a, b as one complex line z = x_a + i x_b, from their half spectra X_a, X_b
// (read for k < kk, zero beyond): Z[k] = X_a[k] + i X_b[k] and Z[N-k] = conj X_a[k] + i conj X_b[k]
// for 0 < k < N/2; the imaginary parts of the k = 0 and k = N/2 terms are dropped (the c2r of
// fftw.f90:73-103 ignores them).  The unnormalised inverse FFT of Z then gives both rows.
template <class T, int N>
__device__ __forceinline__ void pair_c2r(typename Store<T>::C* z, int t, int kk, const typename Store<T>::C* __restrict__ xa,
                                         const typename Store<T>::C* __restrict__ xb) {
  constexpr int TPL = Plan<N>::TPL;
  auto put = [&](int k, cx<T> a, cx<T> b) {
    if (k == 0 || 2 * k == N) {
      Store<T>::stc(z + sm_idx<1>(k), cx<T>{a.re, b.re});
    } else {
      Store<T>::stc(z + sm_idx<1>(k), cx<T>{a.re - b.im, a.im + b.re});
      Store<T>::stc(z + sm_idx<1>(N - k), cx<T>{a.re + b.im, b.re - a.im});
    }
  };
  if constexpr (sizeof(typename Store<T>::C) == 8) {  // FP32 lines: all loads first
    constexpr int NIT = (N / 2 + TPL) / TPL;
    cx<T> va[NIT], vb[NIT];
#pragma unroll
    for (int i = 0; i < NIT; i++) {
      const int k = t + i * TPL;
      const bool in = k <= N / 2 && k < kk;
      va[i] = in ? Store<T>::ldg(xa + k) : cx_zero<T>();
      vb[i] = in ? Store<T>::ldg(xb + k) : cx_zero<T>();
    }
#pragma unroll
    for (int i = 0; i < NIT; i++) {
      const int k = t + i * TPL;
      if (k <= N / 2) put(k, va[i], vb[i]);
    }
  } else {
    for (int k = t; k <= N / 2; k += TPL) {
      const bool in = k < kk;
      put(k, in ? Store<T>::ldg(xa + k) : cx_zero<T>(), in ? Store<T>::ldg(xb + k) : cx_zero<T>());
    }
  }
}

// The two rows' half spectra from the forward FFT Z of z = x_a + i x_b:
// X_a[k] = (Z[k] + conj Z[N-k]) / 2, X_b[k] = (Z[k] - conj Z[N-k]) / 2i, each times 2^scale_exp,
// written for k < kk (k <= N/2).
template <class T, int N>
__device__ __forceinline__ void pair_r2c(const typename Store<T>::C* z, int t, int kk, typename Store<T>::C* xa,
                                         typename Store<T>::C* xb, int scale_exp) {
  constexpr int TPL = Plan<N>::TPL;
  for (int k = t; k <= N / 2 && k < kk; k += TPL) {
    const cx<T> A = Store<T>::ldc(z + sm_idx<1>(k)), B = Store<T>::ldc(z + sm_idx<1>((N - k) & (N - 1)));
    const cx<T> s = {A.re + B.re, A.im - B.im}, d = {A.im + B.im, B.re - A.re};
    Store<T>::stc(xa + k, cx<T>{Real<T>::mul_pow2(s.re, scale_exp - 1), Real<T>::mul_pow2(s.im, scale_exp - 1)});
    Store<T>::stc(xb + k, cx<T>{Real<T>::mul_pow2(d.re, scale_exp - 1), Real<T>::mul_pow2(d.im, scale_exp - 1)});
  }
}

// r2c post-processing of one line: X[k] = (Z[k] + conj Z[h-k])/2 - i W^k (Z[k] - conj Z[h-k])/2,
// X[0] = Re Z0 + Im Z0, X[h] = Re Z0 - Im Z0; each result times 2^scale_exp, handed to `stx`.
template <class T, int H, class STX>
__device__ __forceinline__ void r2c_post(const typename Store<T>::C* z, int t, STX stx, int scale_exp,
                                         const typename Store<T>::C* __restrict__ twx) {
  constexpr int TPL = Plan<H>::TPL;
  for (int k = t; k <= H / 2; k += TPL) {
    if (k == 0) {
      cx<T> z0 = Store<T>::ldc(z);
      cx<T> x0 = {Real<T>::mul_pow2(z0.re + z0.im, scale_exp), Real<T>::cst(0.0)};
      cx<T> xh = {Real<T>::mul_pow2(z0.re - z0.im, scale_exp), Real<T>::cst(0.0)};
      stx(0, x0);
      stx(H, xh);
      continue;
    }
    int k2 = H - k;
    cx<T> a = Store<T>::ldc(z + sm_idx<1>(k)), b = Store<T>::ldc(z + sm_idx<1>(k2));
    cx<T> wa = Store<T>::ldg(twx + k);
    cx<T> xa = (a + conj(b)) - times_i(wa * (a - conj(b)));
    xa = {Real<T>::mul_pow2(xa.re, scale_exp - 1), Real<T>::mul_pow2(xa.im, scale_exp - 1)};
    stx(k, xa);
    if (k2 != k) {
      cx<T> wb = Store<T>::ldg(twx + k2);
      cx<T> xb = (b + conj(a)) - times_i(wb * (b - conj(a)));
      xb = {Real<T>::mul_pow2(xb.re, scale_exp - 1), Real<T>::mul_pow2(xb.im, scale_exp - 1)};
      stx(k2, xb);
    }
  }
}

// Plain r2c along x: real rows (f, z, y) -> half spectrum rows, times 2^scale_exp.
template <class T, int NX>
__global__ void __launch_bounds__(128) k_row_r2c(const typename Store<T>::R* __restrict__ in, typename Store<T>::C* __restrict__ out,
                                                 long long nrows, int kxp, int scale_exp, const typename Store<T>::C* __restrict__ twx) {
  using RP = RowP<NX>;
  using C = typename Store<T>::C;
  using SR = typename Store<T>::R;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* sc = reinterpret_cast<C*>(smem_raw);
  SR* sr = reinterpret_cast<SR*>(smem_raw);
  long long row0 = (long long)blockIdx.x * RP::LB;
  for (int i = threadIdx.x; i < RP::LB * NX; i += blockDim.x) {
    int l = i / NX, x = i % NX;
    long long r = row0 + l;
    sr[2 * l * RP::LC + row_real_idx(x)] = r < nrows ? in[r * NX + x] : SR{};
  }
  __syncthreads();
  int l = threadIdx.x / RP::TPL, t = threadIdx.x % RP::TPL;
  bool act = l < RP::LB;
  C* z = sc + (act ? l : 0) * RP::LC;
  fft_lines<T, RP::H, -1, 1, 0>(z, 0, t, act, twx, 2);
  long long r = row0 + l;
  if (!act || r >= nrows) return;
  C* o = out + r * kxp;
  r2c_post<T, RP::H>(z, t, [&](int k, cx<T> v) { Store<T>::stc(o + k, v); }, scale_exp, twx);
}

// Plain c2r along x (unnormalised): half spectrum rows -> real rows.
template <class T, int NX>
__global__ void __launch_bounds__(128) k_row_c2r(const typename Store<T>::C* __restrict__ in, typename Store<T>::R* __restrict__ out,
                                                 long long nrows, int kxp, const typename Store<T>::C* __restrict__ twx) {
  using RP = RowP<NX>;
  using C = typename Store<T>::C;
  using SR = typename Store<T>::R;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* sc = reinterpret_cast<C*>(smem_raw);
  SR* sr = reinterpret_cast<SR*>(smem_raw);
  long long row0 = (long long)blockIdx.x * RP::LB;
  int l = threadIdx.x / RP::TPL, t = threadIdx.x % RP::TPL;
  bool act = l < RP::LB && row0 + l < nrows;
  C* z = sc + (l < RP::LB ? l : 0) * RP::LC;
  if (act) {
    const C* x = in + (row0 + l) * kxp;
    c2r_pre<T, RP::H>(z, t, [&](int k) { return Store<T>::ldg(x + k); }, twx);
  }
  __syncthreads();
  fft_lines<T, RP::H, +1, 1, 0>(z, 0, t, l < RP::LB, twx, 2);
  for (int i = threadIdx.x; i < RP::LB * NX; i += blockDim.x) {
    int ll = i / NX, x = i % NX;
    long long r = row0 + ll;
    if (r < nrows) out[r * NX + x] = sr[2 * ll * RP::LC + row_real_idx(x)];
  }
}

// --------------------------------------------------------------------------- pointwise
// primitive (rho, u, B, p) or conserved doubles -> conserved T; mhdinit.f90:1038-1056
template <class T>
__global__ void k_upload_convert(const double* __restrict__ h, typename Store<T>::R* __restrict__ u, long long n, int primitive,
                                 double gamma, int incomp) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double v[8];
#pragma unroll
    for (int f = 0; f < 8; f++) v[f] = h[f * n + i];
    if (primitive) {
      double ux = v[1], uy = v[2], uz = v[3], p = v[7];
      v[1] = v[0] * ux;
      v[2] = v[0] * uy;
      v[3] = v[0] * uz;
      // the incompressible state keeps p in slot 8 (src_incompressible/mhdinit.f90:1031-1042)
      if (!incomp) v[7] = p / (gamma - 1) + 0.5 * (v[0] * (ux * ux + uy * uy + uz * uz) + v[4] * v[4] + v[5] * v[5] + v[6] * v[6]);
    }
#pragma unroll
    for (int f = 0; f < 8; f++) Store<T>::st(u + f * n + i, Real<T>::from_d(v[f]));
  }
}

// one field f of the conversion above, for the pipelined upload (the fields it reads - rho
// for the momentum, all eight for the energy - have arrived)
template <class T>
__global__ void k_upload_field(const double* __restrict__ h, typename Store<T>::R* __restrict__ u, long long n, int f,
                               int primitive, double gamma, int incomp) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double v = h[f * n + i];
    if (primitive) {
      if (f >= 1 && f <= 3) {
        v = h[i] * v;
      } else if (f == 7 && !incomp) {
        const double rho = h[i], ux = h[n + i], uy = h[2 * n + i], uz = h[3 * n + i];
        const double bx = h[4 * n + i], by = h[5 * n + i], bz = h[6 * n + i];
        v = v / (gamma - 1) + 0.5 * (rho * (ux * ux + uy * uy + uz * uz) + bx * bx + by * by + bz * bz);
      }
    }
    Store<T>::st(u + f * n + i, Real<T>::from_d(v));
  }
}

// real T field -> float64 (the conserved fields of the pipelined download)
// FP64 <-> float-float, for the FP64-state transforms of the FP32-transform engine, which run
// in float-float: the bit-field conversions of arith.cuh and one FP64 subtraction or addition
// per value (a value keeps 48 significand bits).  n values; in place allowed (same bytes).
static __global__ void k_f64_to_dd(const double* in, float2* out, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double x = in[i];
    const float hi = f64_to_f32_rn(x);
    const float lo = f64_to_f32_rn(x - f32_to_f64_bits(hi));
    const dd v = dd_fast_two_sum(hi, lo);
    out[i] = make_float2(v.hi, v.lo);
  }
}
static __global__ void k_dd_to_f64(const float2* in, double* out, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float2 v = in[i];
    out[i] = f32_to_f64_bits(v.x) + f32_to_f64_bits(v.y);
  }
}

template <class T>
__global__ void k_field_to_double(const typename Store<T>::R* __restrict__ u, double* __restrict__ h, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    h[i] = Real<T>::to_d(Store<T>::ld(u + i));
}

// conserved T -> conserved doubles + primitives (ux, uy, uz, p); mhdrhs.f90:282-294
template <class T>
__global__ void k_download_convert(const typename Store<T>::R* __restrict__ u, double* __restrict__ h, double* __restrict__ hp,
                                   long long n, double gamma, int incomp) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double v[8];
#pragma unroll
    for (int f = 0; f < 8; f++) v[f] = Real<T>::to_d(Store<T>::ld(u + f * n + i));
    if (h) {
#pragma unroll
      for (int f = 0; f < 8; f++) h[f * n + i] = v[f];
    }
    if (hp) {
      double ux = v[1] / v[0], uy = v[2] / v[0], uz = v[3] / v[0];
      hp[0 * n + i] = ux;
      hp[1 * n + i] = uy;
      hp[2 * n + i] = uz;
      hp[3 * n + i] = incomp ? v[7] : (v[7] - 0.5 * (v[1] * ux + v[2] * uy + v[3] * uz + v[4] * v[4] + v[5] * v[5] + v[6] * v[6])) * (gamma - 1);
    }
  }
}

// spectral copy with the padded pitch <-> the reference's (nx/2+1, ny, nz, 8) complex128
template <class T>
__global__ void k_spec_to_ref(const typename Store<T>::C* __restrict__ U, double2* __restrict__ out, Geo g, int nf) {
  long long tot = (long long)nf * g.nz * g.ny * g.nh;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot; i += (long long)gridDim.x * blockDim.x) {
    int kx = i % g.nh;
    long long r = i / g.nh;  // (f, z, y)
    cx<T> v = Store<T>::ldc(U + r * g.kxp + kx);
    out[i] = make_double2(Real<T>::to_d(v.re), Real<T>::to_d(v.im));
  }
}
template <class T>
__global__ void k_spec_from_ref(const double2* __restrict__ in, typename Store<T>::C* __restrict__ U, Geo g, int nf) {
  long long tot = (long long)nf * g.nz * g.ny * g.kxp;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot; i += (long long)gridDim.x * blockDim.x) {
    int kx = i % g.kxp;
    long long r = i / g.kxp;
    cx<T> v = cx_zero<T>();
    if (kx < g.nh) {
      double2 d = in[r * g.nh + kx];
      v = {Real<T>::from_d(d.x), Real<T>::from_d(d.y)};
    }
    Store<T>::stc(U + i, v);
  }
}

// U += scale * in for nf fields, `in` in the reference's (nx/2+1, ny, nz) complex layout
template <class T>
__global__ void k_spec_axpy_ref(const double2* __restrict__ in, typename Store<T>::C* U, Geo g, int nf, double scale) {
  long long tot = (long long)nf * g.nz * g.ny * g.nh;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot; i += (long long)gridDim.x * blockDim.x) {
    const int kx = (int)(i % g.nh);
    const long long r = i / g.nh;
    typename Store<T>::C* u = U + r * g.kxp + kx;
    const double2 d = in[i];
    const cx<T> v = Store<T>::ldc(u);
    Store<T>::stc(u, v + cx<T>{Real<T>::from_d(scale * d.x), Real<T>::from_d(scale * d.y)});
  }
}

// --------------------------------------------------------------------------- tables / scalars
// Rebuild the wave-number tables for radius R (evolve_radius / update_ksquare,
// AEBmod.f90:56-73,87-125; derivative factors of mhdrhs.f90:191-204).
template <class T>
__global__ void k_tables(const double* __restrict__ wxd, const double* __restrict__ wyd, const double* __restrict__ wzd,
                         typename Store<T>::R* wx, typename Store<T>::R* kxd, typename Store<T>::R* wy, typename Store<T>::R* kyd,
                         typename Store<T>::R* kzd, typename Store<T>::R* kx2, typename Store<T>::R* ky2,
                         typename Store<T>::R* kz2, int nh, int ny, int nz, double R0, int zrad, const StepState* st) {
  double R = st->radius;
  int plain = st->ksq_plain;
  for (int i = threadIdx.x; i < nh; i += blockDim.x) {
    double k = wxd[i];
    double kd = zrad ? k * R0 / R : k;  // src_compressible/2D/mhdrhs.f90:278-280
    Store<T>::st(wx + i, Real<T>::from_d(k));
    Store<T>::st(kxd + i, Real<T>::from_d(kd));
    Store<T>::st(kx2 + i, Real<T>::from_d(plain ? k * k : kd * kd));
  }
  for (int i = threadIdx.x; i < ny; i += blockDim.x) {
    double k = wyd[i];
    double kd = k * R0 / R;
    Store<T>::st(wy + i, Real<T>::from_d(k));
    Store<T>::st(kyd + i, Real<T>::from_d(kd));
    Store<T>::st(ky2 + i, Real<T>::from_d(plain ? k * k : kd * kd));
  }
  for (int i = threadIdx.x; i < nz; i += blockDim.x) {
    double k = wzd[i];
    double kd = k * R0 / R;
    Store<T>::st(kzd + i, Real<T>::from_d(kd));
    Store<T>::st(kz2 + i, Real<T>::from_d(plain ? k * k : kd * kd));
  }
}

// vardt tail: dt = cfl * min, kept within +-2 %, floor check, rkt_init coefficients
// (mhd.f90:418-428, rktmod.f90:15-27).
// The 2-D code recomputes dt only every dstep steps and may forbid increases
// (src_compressible/2D/mhd.f90:237-240,396-405).  force: an explicit laps_vardt call.
static __global__ void k_finalize_dt(StepState* st, double cfl, int dstep, int limit_dt, int force) {
  if (threadIdx.x | blockIdx.x) return;
  if (st->halt) return;
  double m = __longlong_as_double((long long)st->cfl_bits);
  st->cfl_bits = 0x7FF0000000000000ull;  // +inf for the next reduction
  st->cfl32_bits = 0x7F800000u;
  if (!force && dstep > 1 && st->istep % dstep != 0) return;
  double dtmin = m * cfl;
  double dt = st->dt;
  if (limit_dt) {
    if (dt == 0.0 || dt > 1.02 * dtmin) dt = dtmin;
  } else if (dt < 0.98 * dtmin || dt > 1.02 * dtmin) {
    dt = dtmin;
  }
  st->dt = dt;
  st->cc[0] = 8.0 / 15.0 * dt; st->ddc[0] = 0.0;
  st->cc[1] = 5.0 / 12.0 * dt; st->ddc[1] = -17.0 / 60.0 * dt;
  st->cc[2] = 0.75 * dt;       st->ddc[2] = -5.0 / 12.0 * dt;
  st->ts[0] = 8.0 / 15.0 * dt;
  st->ts[1] = 2.0 / 15.0 * dt;
  st->ts[2] = 1.0 / 3.0 * dt;
  step_state_f32(*st);
  if (dt < 0.00000001) {
    st->status |= LAPS_STATUS_DT_FLOOR;
    st->halt = 1;
  }
}

// update_rho_p (3-D incompressible, src_incompressible/AEBmod.f90:123-134, at the step's
// start radius); time += dt; R = R0 + Ur t; tau = R/Ur (mhd.f90:246-248, AEBmod.f90:46-73)
static __global__ void k_advance_time(StepState* st, double R0, double Ur, int incomp) {
  if (threadIdx.x | blockIdx.x) return;
  if (st->halt) return;
  if (incomp) {
    double f = R0 / st->radius;
    st->rho0 = st->rho0 * (f * f);
  }
  st->istep = st->istep + 1;
  st->time = st->time + st->dt;
  st->radius = R0 + Ur * st->time;
  st->inv_tau = Ur != 0.0 ? 1.0 / (st->radius / Ur) : 0.0;
  st->r_ratio = R0 / st->radius;
  st->ksq_plain = 0;
  step_state_f32(*st);
}

}  // namespace laps
