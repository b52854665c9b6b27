// Diagnostics reductions: calc_rms (src_compressible/mhdrms.f90:53-126), calc_max_divB
// (src_compressible/mhd.f90:522-570), and the engine's energy / cross-helicity /
// magnetic-helicity sums.  Each block writes its partial results; the host adds the
// partials in block order, so repeated calls give bitwise-identical results.
#pragma once
#include "kernels.cuh"
#include "passes.cuh"

namespace laps {

template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* out) {
  __shared__ double red[8][NV];
#pragma unroll
  for (int k = 0; k < NV; k++)
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0)
    for (int k = 0; k < NV; k++) red[w][k] = v[k];
  __syncthreads();
  if (threadIdx.x < NV) {
    double s = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) s += red[i][threadIdx.x];
    out[threadIdx.x] = s;
  }
}

// sums of rho, ux, uy, uz, Bx, By, Bz, p, their squares, rho u^2, B^2 and u.B
template <class T>
__global__ void __launch_bounds__(256) k_diag_sums(const typename Store<T>::R* __restrict__ u, long long n, double gamma,
                                                   int incomp, double* part) {
  double v[19];
#pragma unroll
  for (int k = 0; k < 19; k++) v[k] = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double q[8];
#pragma unroll
    for (int f = 0; f < 8; f++) q[f] = Real<T>::to_d(Store<T>::ld(u + f * n + i));
    double ux = q[1] / q[0], uy = q[2] / q[0], uz = q[3] / q[0];
    // the incompressible state holds p itself in slot 8; the reference's rms there reads
    // uu_prim(:,:,:,4) beyond its 3 components (src_incompressible/mhdrms.f90:73,83)
    double p = incomp ? q[7] : (q[7] - 0.5 * (q[1] * ux + q[2] * uy + q[3] * uz + q[4] * q[4] + q[5] * q[5] + q[6] * q[6])) * (gamma - 1);
    double f8[8] = {q[0], ux, uy, uz, q[4], q[5], q[6], p};
#pragma unroll
    for (int k = 0; k < 8; k++) {
      v[k] += f8[k];
      v[8 + k] += f8[k] * f8[k];
    }
    v[16] += q[0] * (ux * ux + uy * uy + uz * uz);
    v[17] += q[4] * q[4] + q[5] * q[5] + q[6] * q[6];
    v[18] += ux * q[4] + uy * q[5] + uz * q[6];
  }
  block_sum<19>(v, part + (size_t)blockIdx.x * 32);
}

// sum of rho (u_i - <u_i>)^2 (mhdrms.f90:110-125)
template <class T>
__global__ void __launch_bounds__(256) k_diag_rhou2(const typename Store<T>::R* __restrict__ u, long long n, double a1, double a2,
                                                    double a3, double* part) {
  double v[3] = {0, 0, 0};
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double rho = Real<T>::to_d(Store<T>::ld(u + i));
    double ux = Real<T>::to_d(Store<T>::ld(u + n + i)) / rho;
    double uy = Real<T>::to_d(Store<T>::ld(u + 2 * n + i)) / rho;
    double uz = Real<T>::to_d(Store<T>::ld(u + 3 * n + i)) / rho;
    v[0] += rho * (ux - a1) * (ux - a1);
    v[1] += rho * (uy - a2) * (uy - a2);
    v[2] += rho * (uz - a3) * (uz - a3);
  }
  block_sum<3>(v, part + (size_t)blockIdx.x * 8);
}

// max |i k.B| and <A.B> with A = i k x B / |k|^2 from the half spectrum (Parseval weights:
// 2 for 0 < kx < nx/2, else 1)
template <class T>
__global__ void __launch_bounds__(256) k_diag_spec(const typename Store<T>::C* __restrict__ U, Geo g, KTab<T> K, Phys P, PT<T> pc,
                                                   const StepState* st, double* part) {
  double mx = 0.0, hm = 0.0;
  long long tot = (long long)g.nz * g.ny * g.nh;
  T rr = Real<T>::from_d(st->r_ratio);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot; i += (long long)gridDim.x * blockDim.x) {
    int kx = i % g.nh;
    long long r = i / g.nh;
    int ky = r % g.ny, kz = r / g.ny;
    long long idx = (long long)kz * g.ny * g.kxp + (long long)ky * g.kxp + kx;
    T axT, ayT, azT;
    kfac(K, P, pc, rr, kx, ky, kz, axT, ayT, azT);
    double ax = Real<T>::to_d(axT), ay = Real<T>::to_d(ayT), az = Real<T>::to_d(azT);
    cx<T> bxT = Store<T>::ldc(U + 4 * g.fsc + idx), byT = Store<T>::ldc(U + 5 * g.fsc + idx), bzT = Store<T>::ldc(U + 6 * g.fsc + idx);
    double bxr = Real<T>::to_d(bxT.re), bxi = Real<T>::to_d(bxT.im);
    double byr = Real<T>::to_d(byT.re), byi = Real<T>::to_d(byT.im);
    double bzr = Real<T>::to_d(bzT.re), bzi = Real<T>::to_d(bzT.im);
    // i (ax Bx + ay By + az Bz)
    double dr = ax * bxr + ay * byr + az * bzr, di = ax * bxi + ay * byi + az * bzi;
    mx = fmax(mx, hypot(dr, di));
    double k2 = ax * ax + ay * ay + az * az;
    if (k2 > 0.0) {
      // c = k x B ; A = i c / k2 ; Re(A . conj B) = -Im(c . conj B) / k2
      double cxr = ay * bzr - az * byr, cxi = ay * bzi - az * byi;
      double cyr = az * bxr - ax * bzr, cyi = az * bxi - ax * bzi;
      double czr = ax * byr - ay * bxr, czi = ax * byi - ay * bxi;
      double im = (cxi * bxr - cxr * bxi) + (cyi * byr - cyr * byi) + (czi * bzr - czr * bzi);
      double w = (kx == 0 || 2 * kx == g.nx) ? 1.0 : 2.0;
      hm += -w * im / k2;
    }
  }
  __shared__ double rm[8];
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) rm[threadIdx.x >> 5] = mx;
  double v[1] = {hm};
  block_sum<1>(v, part + (size_t)blockIdx.x * 2 + 1);
  if (threadIdx.x == 0) {
    double m = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) m = fmax(m, rm[i]);
    part[(size_t)blockIdx.x * 2] = m;
  }
}

// i (ax X + ay Y + az Z) * scale of three state slots, written with the spectral pitch:
// div B (slots 4..6) or div(rho u) / rho0 (slots 1..3) before the inverse transform of
// calc_divB_real / calc_divV_real (src_incompressible/mhdrhs.f90:532-648)
template <class T>
__global__ void k_spec_div(const typename Store<T>::C* __restrict__ U, typename Store<T>::C* __restrict__ out, Geo g, KTab<T> K,
                           Phys P, PT<T> pc, const StepState* st, int first, int scale_by_rho0) {
  long long tot = (long long)g.nz * g.ny * g.kxp;
  T rr = Real<T>::from_d(st->r_ratio);
  T sc = Real<T>::from_d(scale_by_rho0 ? 1.0 / st->rho0 : 1.0);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot; i += (long long)gridDim.x * blockDim.x) {
    int kx = i % g.kxp;
    long long r = i / g.kxp;
    int ky = r % g.ny, kz = r / g.ny;
    cx<T> v = cx_zero<T>();
    if (kx < g.nh) {
      T ax, ay, az;
      kfac(K, P, pc, rr, kx, ky, kz, ax, ay, az);
      v = (mul_i(Store<T>::ldc(U + first * g.fsc + i), ax) + mul_i(Store<T>::ldc(U + (first + 1) * g.fsc + i), ay)) +
          mul_i(Store<T>::ldc(U + (first + 2) * g.fsc + i), az);
      if (scale_by_rho0) v = v * sc;
    }
    Store<T>::stc(out + i, v);
  }
}

// per-block max |x| of one real field
template <class T>
__global__ void __launch_bounds__(256) k_max_abs(const typename Store<T>::R* __restrict__ u, long long n, double* part) {
  double m = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    m = fmax(m, fabs(Real<T>::to_d(Store<T>::ld(u + i))));
  __shared__ double rm[8];
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) rm[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 1; i < (int)(blockDim.x >> 5); i++) m = fmax(m, rm[i]);
    part[blockIdx.x] = fmax(rm[0], m);
  }
}

// u_i = (rho u_i) / rho in place on the real fields 1..3 (field 0 = rho), field pitch n
template <class T>
__global__ void __launch_bounds__(256) k_velocity(typename Store<T>::R* __restrict__ u, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const T r = Store<T>::ld(u + i);
#pragma unroll
    for (int c = 1; c <= 3; c++) Store<T>::st(u + c * n + i, Store<T>::ld(u + c * n + i) / r);
  }
}

// Shell spectra of two 3-component half spectra (pitch `pitch`): 1/2 |u_hat|^2 and
// 1/2 |B_hat|^2 summed over the modes with round(|k| inv_dk) = s < nshell, |k| from the
// unscaled wave numbers, modes 0 < kx < nx/2 counted twice.  Deterministic: a warp adds the
// lanes that share a shell in lane order (__match_any_sync), keeps its own shell array in
// shared memory, and the block adds its 4 warp arrays in order; the host adds the blocks.
constexpr int SPEC_WARPS = 4;
template <class T>
__global__ void __launch_bounds__(SPEC_WARPS * 32) k_shell_spectrum(const typename Store<T>::C* __restrict__ uh,
                                                                    const typename Store<T>::C* __restrict__ bh, long long pitch,
                                                                    Geo g, const double* __restrict__ wx, const double* __restrict__ wy,
                                                                    const double* __restrict__ wz, double inv_dk, int nshell,
                                                                    double* __restrict__ part) {
  extern __shared__ double sh[];  // [SPEC_WARPS][2][nshell]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int i = threadIdx.x; i < SPEC_WARPS * 2 * nshell; i += blockDim.x) sh[i] = 0.0;
  __syncthreads();
  double* mine = sh + warp * 2 * nshell;
  const long long tot = (long long)g.nz * g.ny * g.nh;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long base = (long long)blockIdx.x * blockDim.x + warp * 32; base < tot; base += stride) {
    const long long i = base + lane;
    int key = -1;
    double eu = 0.0, eb = 0.0;
    if (i < tot) {
      const int kx = (int)(i % g.nh);
      const long long r = i / g.nh;
      const int ky = (int)(r % g.ny), kz = (int)(r / g.ny);
      const double kk = sqrt(wx[kx] * wx[kx] + wy[ky] * wy[ky] + wz[kz] * wz[kz]);
      const int s = (int)floor(kk * inv_dk + 0.5);
      if (s < nshell) {
        key = s;
        const long long idx = (long long)kz * g.ny * g.kxp + (long long)ky * g.kxp + kx;
#pragma unroll
        for (int c = 0; c < 3; c++) {
          cx<T> a = Store<T>::ldc(uh + c * pitch + idx), b = Store<T>::ldc(bh + c * pitch + idx);
          double ar = Real<T>::to_d(a.re), ai = Real<T>::to_d(a.im), br = Real<T>::to_d(b.re), bi = Real<T>::to_d(b.im);
          eu += ar * ar + ai * ai;
          eb += br * br + bi * bi;
        }
        const double w = (kx == 0 || 2 * kx == g.nx) ? 0.5 : 1.0;
        eu *= w;
        eb *= w;
      }
    }
    const unsigned m = __match_any_sync(0xffffffffu, key);
    double su = 0.0, sb = 0.0;
    for (int l = 0; l < 32; l++) {
      const double xu = __shfl_sync(0xffffffffu, eu, l), xb = __shfl_sync(0xffffffffu, eb, l);
      if ((m >> l) & 1u) {
        su += xu;
        sb += xb;
      }
    }
    if (key >= 0 && lane == __ffs(m) - 1) {
      mine[key] += su;
      mine[nshell + key] += sb;
    }
  }
  __syncthreads();
  for (int s = threadIdx.x; s < 2 * nshell; s += blockDim.x) {
    double acc = 0.0;
    for (int w = 0; w < SPEC_WARPS; w++) acc += sh[w * 2 * nshell + s];
    part[(size_t)blockIdx.x * 2 * nshell + s] = acc;
  }
}

// ---------------------------------------------------------------------------- granular path
// One component of J = i k x B (calc_current_density_real, mhdrhs.f90:296-362, with the
// expanding-box / corotation factors of kfac), written with the spectral pitch.
template <class T>
__global__ void k_spec_curl(const typename Store<T>::C* __restrict__ U, typename Store<T>::C* __restrict__ out, Geo g, KTab<T> K,
                            Phys P, PT<T> pc, const StepState* st, int comp) {
  const long long tot = (long long)g.nz * g.ny * g.kxp;
  const T rr = Real<T>::from_d(st->r_ratio);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot; i += (long long)gridDim.x * blockDim.x) {
    const int kx = (int)(i % g.kxp);
    const long long r = i / g.kxp;
    const int ky = (int)(r % g.ny), kz = (int)(r / g.ny);
    cx<T> v = cx_zero<T>();
    if (kx < g.nh) {
      T ax, ay, az;
      kfac(K, P, pc, rr, kx, ky, kz, ax, ay, az);
      const cx<T> bx = Store<T>::ldc(U + 4 * g.fsc + i), by = Store<T>::ldc(U + 5 * g.fsc + i), bz = Store<T>::ldc(U + 6 * g.fsc + i);
      if (comp == 0) v = mul_i(bz, ay) - mul_i(by, az);
      else if (comp == 1) v = mul_i(bx, az) - mul_i(bz, ax);
      else v = mul_i(by, ax) - mul_i(bx, ay);
    }
    Store<T>::stc(out + i, v);
  }
}

// Flux k of calc_flux (mhdrhs.f90:21-124; k = 18: the expansion term of :157-171) at every
// point from the real inputs (state, then J), as float64 or in the state type.
template <class T, bool TO_DOUBLE>
__global__ void k_flux_point(const typename Store<T>::R* __restrict__ in, long long n, int nin, int k, void* out, PT<T> c,
                             Phys P, double inv_tau) {
  const T it = Real<T>::from_d(inv_tau), one = c.one;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    T q[11];
#pragma unroll
    for (int f = 0; f < 11; f++) q[f] = f < nin ? Store<T>::ld(in + f * n + i) : c.zero;
    Flux<T>::eval(q, [&](int kk, T v) {
      if (kk != k) return;
      if constexpr (TO_DOUBLE) static_cast<double*>(out)[i] = Real<T>::to_d(v);
      else Store<T>::st(static_cast<typename Store<T>::R*>(out) + i, v);
    }, c, P, it, one);
  }
}

// the dealias mask or filter applied to the state (dealiasing.f90:70-113)
template <class T>
__global__ void k_dealias_state(typename Store<T>::C* __restrict__ U, Geo g, KTab<T> K, Phys P) {
  const long long tot = 8LL * g.fsc;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot; i += (long long)gridDim.x * blockDim.x) {
    const int kx = (int)(i % g.kxp);
    const long long r = (i / g.kxp) % ((long long)g.ny * g.nz);
    const int ky = (int)(r % g.ny), kz = (int)(r / g.ny);
    if (kx >= g.nh) continue;
    cx<T> v = Store<T>::ldc(U + i);
    if (P.dealias == 1 || P.dealias == 3) {
      if (kx >= K.kxlim[kz * g.ny + ky]) v = cx_zero<T>();
    } else if (P.dealias == 2) {
      v = ((v * K.fx[kx]) * K.fy[ky]) * K.fz[kz];
    }
    Store<T>::stc(U + i, v);
  }
}

}  // namespace laps
