// The five fused passes of one RK stage of the 3-D compressible solver (see kernels.cuh).
#pragma once
#include "kernels.cuh"

namespace laps {

struct PassArgs {
  Geo g;
  Phys P;
  int hall, aeb;
  int stage;       // 0, 1, 2
  int store_rk;    // write fnl_rk (not needed after the last stage of a fused step)
  int cfl;         // pass C computes the CFL minimum
  StepState* st;
};

// tile coordinates shared by the column passes
template <class T, int N> struct ColCtx {
  using CL = Col<T, N>;
  using C = typename Store<T>::C;
  int tl, tid, c, t;
  C* s;
  __device__ ColCtx(C* sm) {
    tl = threadIdx.x / CL::NT;
    tid = threadIdx.x % CL::NT;
    c = tid % TX;
    t = tid / TX;
    s = sm + tl * N * TX;
  }
  __device__ __forceinline__ int j(int m) const { return t + m * CL::TPL; }
  __device__ __forceinline__ C* at(int m) const { return s + j(m) * TX + c; }
};

// ============================================================================ pass A
// inverse z-FFT of the 8 state fields, plus C_x = IFFT_z(-i kz B_y), C_y = IFFT_z(i kz B_x)
// for the Hall current.  Tile: kx0..kx0+7, one kept ky row; writes all z of W1.
template <class T, int NZ>
__global__ void __launch_bounds__(Col<T, NZ>::THREADS) k_passA(Bufs<T> b, PassArgs a, PT<T> pc, KTab<T> K, const typename Store<T>::C* __restrict__ twz) {
  using CL = Col<T, NZ>;
  using C = typename Store<T>::C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  if (a.st->halt) return;
  ColCtx<T, NZ> x(reinterpret_cast<C*>(smem_raw));
  const Geo& g = a.g;
  int kx = blockIdx.x * TX + x.c;
  int r = blockIdx.y * CL::NTILE + x.tl;
  bool ok = kx < g.kx_keep && r < g.nky();
  int ky = ok ? g.ky_of(r) : 0;
  long long col = (long long)ky * g.kxp + kx;  // + z * ny * kxp
  long long zs = (long long)g.ny * g.kxp;
  int nout = a.hall ? 10 : 8;
  for (int f = 0; f < nout; f++) {
    int src = f < 8 ? f : (f == 8 ? 5 : 4);  // Cx from By, Cy from Bx
#pragma unroll 4
    for (int m = 0; m < CL::EPT; m++) {
      int kz = x.j(m);
      cx<T> v = cx_zero<T>();
      if (ok && g.kz_in(kz)) {
        v = Store<T>::ldg(b.U + src * g.fsc + kz * zs + col);
        if (f == 8) v = -mul_i(v, K.kzd[kz]);
        else if (f == 9) v = mul_i(v, K.kzd[kz]);
      }
      Store<T>::stc(x.at(m), v);
    }
    __syncthreads();
    fft_lines<T, NZ, +1, TX, 1>(x.s, x.c, x.t, true, twz, 1);
    if (ok) {
#pragma unroll 4
      for (int m = 0; m < CL::EPT; m++) Store<T>::stc(b.W1 + f * g.fsc + x.j(m) * zs + col, Store<T>::ldc(x.at(m)));
    }
    __syncthreads();
  }
}

// ============================================================================ pass B
// inverse y-FFT of the 8 state fields and of the three Hall current components
//   Jx = i ay W1[Bz] + W1[Cx],  Jy = W1[Cy] - i ax W1[Bz],  Jz = i ax W1[By] - i ay W1[Bx]
// Tile: kx0..kx0+7, one z plane; reads kept ky rows, writes all y of W2.
template <class T, int NY>
__global__ void __launch_bounds__(Col<T, NY>::THREADS) k_passB(Bufs<T> b, PassArgs a, PT<T> pc, KTab<T> K, const typename Store<T>::C* __restrict__ twy) {
  using CL = Col<T, NY>;
  using C = typename Store<T>::C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  if (a.st->halt) return;
  ColCtx<T, NY> x(reinterpret_cast<C*>(smem_raw));
  const Geo& g = a.g;
  int kx = blockIdx.x * TX + x.c;
  int z = blockIdx.y * CL::NTILE + x.tl;
  bool ok = kx < g.kx_keep && z < g.nz;
  long long col = (long long)z * g.ny * g.kxp + kx;  // + y * kxp
  T rr = Real<T>::from_d(a.st->r_ratio);
  int nout = a.hall ? 11 : 8;
  for (int f = 0; f < nout; f++) {
#pragma unroll 4
    for (int m = 0; m < CL::EPT; m++) {
      int ky = x.j(m);
      cx<T> v = cx_zero<T>();
      if (ok && g.ky_in(ky)) {
        const C* w = b.W1 + col + (long long)ky * g.kxp;
        if (f < 8) {
          v = Store<T>::ldg(w + f * g.fsc);
        } else {
          T ax, ay, az;
          kfac(K, a.P, pc, rr, kx, ky, 0, ax, ay, az);
          if (f == 8) v = mul_i(Store<T>::ldg(w + 6 * g.fsc), ay) + Store<T>::ldg(w + 8 * g.fsc);
          else if (f == 9) v = Store<T>::ldg(w + 9 * g.fsc) - mul_i(Store<T>::ldg(w + 6 * g.fsc), ax);
          else v = mul_i(Store<T>::ldg(w + 5 * g.fsc), ax) - mul_i(Store<T>::ldg(w + 4 * g.fsc), ay);
        }
      }
      Store<T>::stc(x.at(m), v);
    }
    __syncthreads();
    fft_lines<T, NY, +1, TX, 1>(x.s, x.c, x.t, true, twy, 1);
    if (ok) {
#pragma unroll 4
      for (int m = 0; m < CL::EPT; m++)
        Store<T>::stc(b.W2 + f * g.fsc + col + (long long)x.j(m) * g.kxp, Store<T>::ldc(x.at(m)));
    }
    __syncthreads();
  }
}

// ============================================================================ pass C
// Per x-row (y, z): c2r of the 8 (+3) fields, the real-space fluxes of calc_flux
// (mhdrhs.f90:21-124, with the primitives of update_uu_prim_from_uu, :282-294), the CFL
// minimum of vardt (mhd.f90:350-416) when asked, and r2c of the 18 (+1) fluxes.
template <class T>
struct Flux {
  // in: rho, mx, my, mz, Bx, By, Bz, e, Jx, Jy, Jz ; out: 18 fluxes + expansion term
  __device__ __forceinline__ static void eval(const T* q, T* f, const PT<T>& c, int hall, int aeb, T inv_tau) {
    const T half = c.half, gm1 = c.gm1;
    T rho = q[0], mx = q[1], my = q[2], mz = q[3], Bx = q[4], By = q[5], Bz = q[6], e = q[7];
    T rinv = c.one / rho;
    T ux = mx * rinv, uy = my * rinv, uz = mz * rinv;
    T b2 = Bx * Bx + By * By + Bz * Bz;
    T p = (e - half * (mx * ux + my * uy + mz * uz + b2)) * gm1;
    T ptot = p + half * b2;
    T udotb = ux * Bx + uy * By + uz * Bz;
    f[0] = mx; f[1] = my; f[2] = mz;
    f[3] = mx * ux - Bx * Bx + ptot;
    f[4] = my * ux - By * Bx;
    f[5] = mz * ux - Bz * Bx;
    f[6] = mx * uy - Bx * By;
    f[7] = my * uy - By * By + ptot;
    f[8] = mz * uy - Bz * By;
    f[9] = mx * uz - Bx * Bz;
    f[10] = my * uz - By * Bz;
    f[11] = mz * uz - Bz * Bz + ptot;
    f[12] = uz * By - uy * Bz;
    f[13] = ux * Bz - uz * Bx;
    f[14] = uy * Bx - ux * By;
    T ep = e + ptot;
    f[15] = ep * ux - udotb * Bx;
    f[16] = ep * uy - udotb * By;
    f[17] = ep * uz - udotb * Bz;
    if (aeb) {
      T two = c.two;
      f[18] = c.cg * p * inv_tau - (two * Bx * Bx + By * By + Bz * Bz) * inv_tau - (mx * ux + two * my * uy + two * mz * uz) * inv_tau;
    }
    if (hall) {
      T dr = c.di * rinv;
      T Jx = q[8], Jy = q[9], Jz = q[10];
      f[12] = f[12] + dr * (Jy * Bz - Jz * By);
      f[13] = f[13] + dr * (Jz * Bx - Jx * Bz);
      f[14] = f[14] + dr * (Jx * By - Jy * Bx);
    }
  }
  // min over the three axes of dx_i / c_max,i (mhd.f90:355-409)
  __device__ __forceinline__ static T cfl(const T* q, const PT<T>& c, int hall, T rfac) {
    const T zero = c.zero, four = c.four, half = c.half;
    const T is2 = c.is2;
    T rho = q[0], rinv = c.one / rho;
    T ux = q[1] * rinv, uy = q[2] * rinv, uz = q[3] * rinv;
    T Bx = q[4], By = q[5], Bz = q[6];
    T p = (q[7] - half * (q[1] * ux + q[2] * uy + q[3] * uz + Bx * Bx + By * By + Bz * Bz)) * c.gm1;
    T cs2 = c.gamma * p * rinv;
    T sq = Real<T>::sqrt_(rho);
    T ca[3] = {Bx / sq, By / sq, Bz / sq};
    T u[3] = {ux, uy, uz};
    T ca2 = ca[0] * ca[0] + ca[1] * ca[1] + ca[2] * ca[2];
    T cms2 = cs2 + ca2;
    T cmax[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
      T cns = Real<T>::sqrt_(Real<T>::max_(cms2 * cms2 - (four * cs2) * (ca[d] * ca[d]), zero));
      T cf = Real<T>::sqrt_(cms2 + cns) * is2;
      T cs = Real<T>::sqrt_(Real<T>::max_(cms2 - cns, zero)) * is2;
      T m = Real<T>::abs_(u[d] + cf);
      m = Real<T>::max_(m, Real<T>::abs_(u[d] + cs));
      m = Real<T>::max_(m, Real<T>::abs_(u[d] + ca[d]));
      m = Real<T>::max_(m, Real<T>::abs_(u[d] - cf));
      m = Real<T>::max_(m, Real<T>::abs_(u[d] - cs));
      m = Real<T>::max_(m, Real<T>::abs_(u[d] - ca[d]));
      m = Real<T>::max_(m, Real<T>::abs_(u[d]));
      cmax[d] = m;
    }
    if (hall) {
      T bm = Real<T>::max_(Real<T>::max_(Bx, By), Bz);
      T ch = c.di * rinv * bm * c.inv_mindx;
#pragma unroll
      for (int d = 0; d < 3; d++) cmax[d] = Real<T>::max_(cmax[d], ch);
    }
    T dtx = c.dx / cmax[0];
    T dty = c.dy / cmax[1] * rfac;
    T dtz = c.dz / cmax[2] * rfac;
    return Real<T>::min_(Real<T>::min_(dtx, dty), dtz);
  }
};

template <int NX> struct PassCCfg {
  static constexpr int ROWS = NX >= 128 ? 1 : 128 / NX;  // rows per block (ny*nz is a multiple)
  static constexpr int NF = 19;
  static constexpr int PPT = NX * ROWS / 128;  // points per thread (NX >= 128)
};

template <class T, int NX>
__global__ void __launch_bounds__(128) k_passC(Bufs<T> b, PassArgs a, PT<T> pc, const typename Store<T>::C* __restrict__ twx) {
  using RP = RowP<NX>;
  using CF = PassCCfg<NX>;
  using C = typename Store<T>::C;
  using SR = typename Store<T>::R;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double red[4];
  if (a.st->halt) return;
  SR* sr = reinterpret_cast<SR*>(smem_raw);  // [row][field][x]
  const Geo& g = a.g;
  const int nin = a.hall ? 11 : 8;
  const int nfl = a.cfl == 2 ? 0 : (a.aeb ? 19 : 18);
  long long row0 = (long long)blockIdx.x * CF::ROWS;  // row = z*ny + y
  int lt = threadIdx.x % RP::TPL, lb = threadIdx.x / RP::TPL;
  // ---- c2r of the inputs, LB lines per batch
  for (int L0 = 0; L0 < CF::ROWS * nin; L0 += RP::LB) {
    int L = L0 + lb;
    bool act = lb < RP::LB && L < CF::ROWS * nin;
    int rr = act ? L / nin : 0, f = act ? L % nin : 0;
    C* z = reinterpret_cast<C*>(sr + (rr * CF::NF + f) * NX);
    if (act) {
      const C* xin = b.W2 + f * g.fsc + (row0 + rr) * g.kxp;
      int kk = g.kx_keep;
      c2r_pre<T, RP::H>(z, lt, [&](int k) { return k < kk ? Store<T>::ldg(xin + k) : cx_zero<T>(); }, twx);
    }
    __syncthreads();
    fft_lines<T, RP::H, +1, 1, 0>(z, 0, lt, act, twx, 2);
  }
  // ---- physics per point
  T q[CF::PPT][11];
  const T inv_tau = Real<T>::from_d(a.st->inv_tau);
#pragma unroll
  for (int pp = 0; pp < CF::PPT; pp++) {
    int p = threadIdx.x + pp * 128;
    int rr = p / NX, xx = p % NX;
#pragma unroll
    for (int f = 0; f < 11; f++)
      if (f < nin) q[pp][f] = Store<T>::ld(sr + (rr * CF::NF + f) * NX + xx);
  }
  __syncthreads();
  T tmin = Real<T>::inf();
  bool nan_seen = false;
  const T rfac = Real<T>::from_d(a.st->radius / a.P.R0);
#pragma unroll
  for (int pp = 0; pp < CF::PPT; pp++) {
    int p = threadIdx.x + pp * 128;
    int rr = p / NX, xx = p % NX;
    if (a.cfl) {
      T d = Flux<T>::cfl(q[pp], pc, a.hall, rfac);
      if (Real<T>::isnan_(d)) nan_seen = true;
      else tmin = Real<T>::min_(tmin, d);
    }
    if (nfl == 0) continue;
    T f[19];
    Flux<T>::eval(q[pp], f, pc, a.hall, a.aeb, inv_tau);
#pragma unroll
    for (int k = 0; k < 19; k++)
      if (k < nfl) Store<T>::st(sr + (rr * CF::NF + k) * NX + xx, f[k]);
  }
  if (a.cfl) {
    double dmin = Real<T>::to_d(tmin);
    for (int o = 16; o > 0; o >>= 1) dmin = fmin(dmin, __shfl_xor_sync(0xffffffffu, dmin, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = dmin;
    if (__any_sync(0xffffffffu, nan_seen) && (threadIdx.x & 31) == 0) atomicOr(&a.st->status, LAPS_STATUS_NAN);
  }
  __syncthreads();
  if (a.cfl && threadIdx.x == 0) {
    double m = fmin(fmin(red[0], red[1]), fmin(red[2], red[3]));
    atomicMin(&a.st->cfl_bits, (unsigned long long)__double_as_longlong(m));
  }
  // ---- r2c of the fluxes
  int sexp = -__ffs(NX) + 1;  // 1/nx
  for (int L0 = 0; L0 < CF::ROWS * nfl; L0 += RP::LB) {
    int L = L0 + lb;
    bool act = lb < RP::LB && L < CF::ROWS * nfl;
    int rr = act ? L / nfl : 0, f = act ? L % nfl : 0;
    C* z = reinterpret_cast<C*>(sr + (rr * CF::NF + f) * NX);
    fft_lines<T, RP::H, -1, 1, 0>(z, 0, lt, act, twx, 2);
    if (act) {
      C* xo = b.W1 + f * g.fsc + (row0 + rr) * g.kxp;
      int kk = g.kx_keep;
      r2c_post<T, RP::H>(z, lt, [&](int k, cx<T> v) { if (k < kk) Store<T>::stc(xo + k, v); }, sexp, twx);
    }
  }
}

// ============================================================================ pass D
// forward y-FFT of the fluxes with the kx, ky parts of the spectral right-hand side folded
// in (calc_rhs, mhdrhs.f90:206-233), leaving only the kz parts for pass E:
//   0 Q1 = -(i ax F1 + i ay F2)      1 F3
//   2 Q2 = -(i ax F4 + i ay F5)      3 F6
//   4 Q3 = -(i ax F7 + i ay F8)      5 F9
//   6 Q4 = -(i ax F10 + i ay F11)    7 F12
//   8 Ex   9 Ey   10 P7 = i ay Ex - i ax Ey   11 P5 = -i ay Ez   12 P6 = i ax Ez
//   13 Q8 = -(i ax F16 + i ay F17) + Expand   14 F18
// Tile: kx0..kx0+7, one z plane; reads all y of W1, writes kept ky rows of W2.
// one forward y-FFT of input `in`, then action `act` with output slots o1, o2
struct DOp { signed char in, act, o1, o2; };
enum { D_ACC_MX = 0, D_ACC_MY_ST, D_ACC_MY, D_ACC_ADD_ST, D_ST, D_EX, D_EY, D_EZ };
__constant__ DOp c_dprog[2][20] = {
    // without the expansion term
    {{0, D_ACC_MX, 0, 0}, {1, D_ACC_MY_ST, 0, 0}, {2, D_ST, 1, 0},
     {3, D_ACC_MX, 0, 0}, {4, D_ACC_MY_ST, 2, 0}, {5, D_ST, 3, 0},
     {6, D_ACC_MX, 0, 0}, {7, D_ACC_MY_ST, 4, 0}, {8, D_ST, 5, 0},
     {9, D_ACC_MX, 0, 0}, {10, D_ACC_MY_ST, 6, 0}, {11, D_ST, 7, 0},
     {12, D_EX, 8, 0}, {13, D_EY, 9, 10}, {14, D_EZ, 11, 12},
     {15, D_ACC_MX, 0, 0}, {16, D_ACC_MY_ST, 13, 0}, {17, D_ST, 14, 0}, {-1, 0, 0, 0}, {-1, 0, 0, 0}},
    // with the expansion term (input 18) added to output 13
    {{0, D_ACC_MX, 0, 0}, {1, D_ACC_MY_ST, 0, 0}, {2, D_ST, 1, 0},
     {3, D_ACC_MX, 0, 0}, {4, D_ACC_MY_ST, 2, 0}, {5, D_ST, 3, 0},
     {6, D_ACC_MX, 0, 0}, {7, D_ACC_MY_ST, 4, 0}, {8, D_ST, 5, 0},
     {9, D_ACC_MX, 0, 0}, {10, D_ACC_MY_ST, 6, 0}, {11, D_ST, 7, 0},
     {12, D_EX, 8, 0}, {13, D_EY, 9, 10}, {14, D_EZ, 11, 12},
     {15, D_ACC_MX, 0, 0}, {16, D_ACC_MY, 0, 0}, {18, D_ACC_ADD_ST, 13, 0}, {17, D_ST, 14, 0}, {-1, 0, 0, 0}}};

template <class T, int NY>
__global__ void __launch_bounds__(Col<T, NY>::THREADS) k_passD(Bufs<T> b, PassArgs a, PT<T> pc, KTab<T> K, const typename Store<T>::C* __restrict__ twy) {
  using CL = Col<T, NY>;
  using C = typename Store<T>::C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  if (a.st->halt) return;
  ColCtx<T, NY> x(reinterpret_cast<C*>(smem_raw));
  const Geo& g = a.g;
  int kx = blockIdx.x * TX + x.c;
  int z = blockIdx.y * CL::NTILE + x.tl;
  bool ok = kx < g.kx_keep && z < g.nz;
  long long col = (long long)z * g.ny * g.kxp + kx;
  T rr = Real<T>::from_d(a.st->r_ratio);
  const int sexp = -__ffs(NY) + 1;
  const DOp* prog = c_dprog[a.aeb ? 1 : 0];
  cx<T> acc[CL::EPT];
  for (int s = 0; s < 20; s++) {
    DOp op = prog[s];
    if (op.in < 0) break;
#pragma unroll 4
    for (int m = 0; m < CL::EPT; m++) {
      cx<T> v = ok ? Store<T>::ldg(b.W1 + op.in * g.fsc + col + (long long)x.j(m) * g.kxp) : cx_zero<T>();
      Store<T>::stc(x.at(m), v);
    }
    __syncthreads();
    fft_lines<T, NY, -1, TX, 1>(x.s, x.c, x.t, true, twy, 1);
#pragma unroll
    for (int m = 0; m < CL::EPT; m++) {
      int ky = x.j(m);
      cx<T> v = Store<T>::ldc(x.at(m));
      v = {Real<T>::mul_pow2(v.re, sexp), Real<T>::mul_pow2(v.im, sexp)};
      T ax, ay, az;
      kfac(K, a.P, pc, rr, kx, ky, 0, ax, ay, az);
      bool st_ok = ok && g.ky_in(ky);
      C* o1 = b.W2 + op.o1 * g.fsc + col + (long long)ky * g.kxp;
      C* o2 = b.W2 + op.o2 * g.fsc + col + (long long)ky * g.kxp;
      switch (op.act) {
        case D_ACC_MX: acc[m] = -mul_i(v, ax); break;
        case D_ACC_MY: acc[m] = acc[m] - mul_i(v, ay); break;
        case D_ACC_MY_ST: acc[m] = acc[m] - mul_i(v, ay); if (st_ok) Store<T>::stc(o1, acc[m]); break;
        case D_ACC_ADD_ST: acc[m] = acc[m] + v; if (st_ok) Store<T>::stc(o1, acc[m]); break;
        case D_ST: if (st_ok) Store<T>::stc(o1, v); break;
        case D_EX: if (st_ok) Store<T>::stc(o1, v); acc[m] = mul_i(v, ay); break;
        case D_EY: if (st_ok) { Store<T>::stc(o1, v); Store<T>::stc(o2, acc[m] - mul_i(v, ax)); } break;
        default: if (st_ok) { Store<T>::stc(o1, -mul_i(v, ay)); Store<T>::stc(o2, mul_i(v, ax)); } break;
      }
    }
    __syncthreads();
  }
}

// ============================================================================ pass E
// forward z-FFT with the kz parts of the right-hand side, then for each variable: the
// expansion damping (mhdrhs.f90:235-251), explicit diffusion (:253-275), the RK3 update with
// implicit diffusion (rktmod.f90:34-62) and the dealias mask or filter (dealiasing.f90:70-113).
// Tile: kx0..kx0+7, one kept ky row; reads all z of W2, writes kept kz of U (and R).
template <class T, int NZ>
__global__ void __launch_bounds__(Col<T, NZ>::THREADS) k_passE(Bufs<T> b, PassArgs a, PT<T> pc, KTab<T> K, const typename Store<T>::C* __restrict__ twz) {
  using CL = Col<T, NZ>;
  using C = typename Store<T>::C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  if (a.st->halt) return;
  ColCtx<T, NZ> x(reinterpret_cast<C*>(smem_raw));
  const Geo& g = a.g;
  const Phys& P = a.P;
  int kx = blockIdx.x * TX + x.c;
  int r = blockIdx.y * CL::NTILE + x.tl;
  bool ok = kx < g.kx_keep && r < g.nky();
  int ky = ok ? g.ky_of(r) : 0;
  long long col = (long long)ky * g.kxp + kx;
  long long zs = (long long)g.ny * g.kxp;
  T rr = Real<T>::from_d(a.st->r_ratio);
  const int sexp = -__ffs(NZ) + 1;
  const int stg = a.stage;
  const T cc = Real<T>::from_d(a.st->cc[stg]), ddc = Real<T>::from_d(a.st->ddc[stg]);
  const T ts = Real<T>::from_d(a.st->ts[stg]);
  const T inv_tau = Real<T>::from_d(a.st->inv_tau);
  const int plain = a.st->ksq_plain;
  cx<T> acc[CL::EPT];
  // inputs per variable: first (plain), second (times s * i kz), s = +-1 or 0
  const int in1[8] = {0, 2, 4, 6, 11, 12, 10, 13};
  const int in2[8] = {1, 3, 5, 7, 9, 8, -1, 14};
  const int sg2[8] = {-1, -1, -1, -1, +1, -1, 0, -1};
  int v = 0, part = 0;
  for (;;) {
    const T ebmv = pc.ebm[v] * inv_tau;
    int fi = part == 0 ? in1[v] : in2[v];
#pragma unroll 4
    for (int m = 0; m < CL::EPT; m++) {
      cx<T> w = ok ? Store<T>::ldg(b.W2 + fi * g.fsc + x.j(m) * zs + col) : cx_zero<T>();
      Store<T>::stc(x.at(m), w);
    }
    __syncthreads();
    fft_lines<T, NZ, -1, TX, 1>(x.s, x.c, x.t, true, twz, 1);
#pragma unroll
    for (int m = 0; m < CL::EPT; m++) {
      cx<T> w = Store<T>::ldc(x.at(m));
      w = {Real<T>::mul_pow2(w.re, sexp), Real<T>::mul_pow2(w.im, sexp)};
      if (part == 0) acc[m] = w;
      else {
        w = mul_i(w, K.kzd[x.j(m)]);
        acc[m] = sg2[v] > 0 ? acc[m] + w : acc[m] - w;
      }
    }
    __syncthreads();
    if (part == 0 && in2[v] >= 0) { part = 1; continue; }
    part = 0;
    if (ok) {
    // ---- epilogue: RHS tail, RK3, implicit diffusion, dealias
#pragma unroll
    for (int m = 0; m < CL::EPT; m++) {
      int kz = x.j(m);
      if (!g.kz_in(kz)) continue;
      long long idx = kz * zs + col;
      cx<T> fnl = acc[m];
      cx<T> u = Store<T>::ldg(b.U + v * g.fsc + idx);
      T k2 = pc.zero;
      bool need_k2 = (v >= 1 && v <= 3 && P.visc) || (v >= 4 && v <= 6 && P.resis);
      if (need_k2) {
        if (P.corot && !plain) k2 = ksq(K, P, pc, rr, kx, ky, kz);
        else k2 = (K.kx2[kx] + K.ky2[ky]) + K.kz2[kz];
      }
      if (P.aeb && v < 7) fnl = fnl - u * ebmv;
      if (v >= 1 && v <= 3 && P.visc && P.visc_exp) fnl = fnl - u * (pc.nu * k2);
      if (v >= 4 && v <= 6 && P.resis && P.resis_exp && !(P.cons_bg && kx == 0 && kz == 0))
        fnl = fnl - u * (pc.eta * k2);
      cx<T> un = fnl * cc + u;
      if (stg > 0) un = (fnl * cc + Store<T>::ldg(b.R + v * g.fsc + idx) * ddc) + u;
      if (a.store_rk) Store<T>::stc(b.R + v * g.fsc + idx, fnl);
      if (v >= 1 && v <= 3 && P.visc && !P.visc_exp) {
        T d = ts * k2 * pc.nu + pc.one;
        un = {un.re / d, un.im / d};
      }
      if (v >= 4 && v <= 6 && P.resis && !P.resis_exp) {
        T d = ts * k2 * pc.eta + pc.one;
        un = {un.re / d, un.im / d};
      }
      if (P.dealias == 1) {
        int lim = K.kxlim[kz * g.ny + ky];
        if (kx >= lim) un = cx_zero<T>();
      } else if (P.dealias == 2) {
        un = ((un * K.fx[kx]) * K.fy[ky]) * K.fz[kz];
      }
      Store<T>::stc(b.U + v * g.fsc + idx, un);
    }
    }
    if (++v == 8) break;
  }
}

}  // namespace laps
