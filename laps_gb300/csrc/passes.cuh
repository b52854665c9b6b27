// The five fused passes of one RK stage of the 3-D compressible solver (see kernels.cuh).
//
// Column passes (A, B, D, E) spread their fields over blockIdx.z: one CTA transforms one
// tile (TX adjacent columns) of one field group, so each CTA runs 1-3 FFTs and keeps
// partial results in shared-memory buffers, not registers.
#pragma once
#include "kernels.cuh"

namespace laps {

struct PassArgs {
  Geo g;
  Phys P;
  int hall, aeb;
  int stage;       // 0, 1, 2
  int store_rk;    // write fnl_rk (not needed after the last stage of a fused step)
  int cfl;         // pass C: 0 fluxes, 1 fluxes + CFL minimum, 2 CFL minimum only
  StepState* st;
};

// tile coordinates shared by the column passes; NBUF shared-memory buffers per tile
template <class T, int N, int NBUF> struct ColCtx {
  using CL = Col<T, N>;
  using C = typename Store<T>::C;
  int tl, tid, c, t;
  C* s;
  __device__ ColCtx(C* sm) {
    tl = threadIdx.x / CL::NT;
    tid = threadIdx.x % CL::NT;
    c = tid % TX;
    t = tid / TX;
    s = sm + tl * NBUF * N * TX;
  }
  __device__ __forceinline__ int j(int m) const { return t + m * CL::TPL; }
  __device__ __forceinline__ C* buf(int b) const { return s + b * N * TX; }
  __device__ __forceinline__ C* at(int b, int m) const { return buf(b) + j(m) * TX + c; }
};

// ============================================================================ pass A
// inverse z-FFT of state field f = blockIdx.z (0..7), or for the Hall current
// f = 8: C_x = IFFT_z(-i kz B_y), f = 9: C_y = IFFT_z(i kz B_x).
// Tile: kx0..kx0+7, one kept ky row; writes all z of W1.
template <class T, int NZ>
__global__ void __launch_bounds__(Col<T, NZ>::THREADS) k_passA(Bufs<T> b, PassArgs a, PT<T> pc, KTab<T> K, const typename Store<T>::C* __restrict__ twz) {
  using CL = Col<T, NZ>;
  using C = typename Store<T>::C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  if (a.st->halt) return;
  ColCtx<T, NZ, 1> x(reinterpret_cast<C*>(smem_raw));
  const Geo& g = a.g;
  const int f = blockIdx.z;
  int kx = blockIdx.x * TX + x.c;
  int r = blockIdx.y * CL::NTILE + x.tl;
  bool ok = kx < g.kx_keep && r < g.nky();
  int ky = ok ? g.ky_of(r) : 0;
  long long col = (long long)ky * g.kxp + kx;  // + z * ny * kxp
  long long zs = (long long)g.ny * g.kxp;
  const int src = f < 8 ? f : (f == 8 ? 5 : 4);
  const C* in = b.U + src * g.fsc + col;
#pragma unroll 4
  for (int m = 0; m < CL::EPT; m++) {
    int kz = x.j(m);
    cx<T> v = cx_zero<T>();
    if (ok && g.kz_in(kz)) {
      v = Store<T>::ldg(in + kz * zs);
      if (f == 8) v = -mul_i(v, K.kzd[kz]);
      else if (f == 9) v = mul_i(v, K.kzd[kz]);
    }
    Store<T>::stc(x.at(0, m), v);
  }
  __syncthreads();
  fft_lines<T, NZ, +1, TX, 1>(x.buf(0), x.c, x.t, true, twz, 1);
  if (!ok) return;
  C* out = b.W1 + f * g.fsc + col;
#pragma unroll 4
  for (int m = 0; m < CL::EPT; m++) Store<T>::stc(out + x.j(m) * zs, Store<T>::ldc(x.at(0, m)));
}

// ============================================================================ pass B
// inverse y-FFT of field f = blockIdx.z: the 8 state fields, and for the Hall current
//   8: Jx = i ay W1[Bz] + W1[Cx],  9: Jy = W1[Cy] - i ax W1[Bz],  10: Jz = i ax W1[By] - i ay W1[Bx]
// Tile: kx0..kx0+7, one z plane; reads kept ky rows, writes all y of W2.
template <class T, int NY>
__global__ void __launch_bounds__(Col<T, NY>::THREADS) k_passB(Bufs<T> b, PassArgs a, PT<T> pc, KTab<T> K, const typename Store<T>::C* __restrict__ twy) {
  using CL = Col<T, NY>;
  using C = typename Store<T>::C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  if (a.st->halt) return;
  ColCtx<T, NY, 1> x(reinterpret_cast<C*>(smem_raw));
  const Geo& g = a.g;
  const int f = blockIdx.z;
  int kx = blockIdx.x * TX + x.c;
  int z = blockIdx.y * CL::NTILE + x.tl;
  bool ok = kx < g.kx_keep && z < g.nz;
  long long col = (long long)z * g.ny * g.kxp + kx;  // + y * kxp
  T rr = Real<T>::from_d(a.st->r_ratio);
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
    Store<T>::stc(x.at(0, m), v);
  }
  __syncthreads();
  fft_lines<T, NY, +1, TX, 1>(x.buf(0), x.c, x.t, true, twy, 1);
  if (!ok) return;
  C* out = b.W2 + f * g.fsc + col;
#pragma unroll 4
  for (int m = 0; m < CL::EPT; m++) Store<T>::stc(out + (long long)x.j(m) * g.kxp, Store<T>::ldc(x.at(0, m)));
}

// ============================================================================ pass C
// Per x-row (y, z): c2r of the 8 (+3) fields, the real-space fluxes of calc_flux
// (mhdrhs.f90:21-124, with the primitives of update_uu_prim_from_uu, :282-294), the CFL
// minimum of vardt (mhd.f90:350-416) when asked, and r2c of the 18 (+1) fluxes.
template <class T>
struct Flux {
  // in: rho, mx, my, mz, Bx, By, Bz, e, Jx, Jy, Jz ; out(k, value) receives the 18 fluxes and
  // the expansion term (k = 18) one at a time, so that they need not all be live at once
  template <class OUT>
  __device__ __forceinline__ static void eval(const T* q, OUT out, const PT<T>& c, int hall, int aeb, T inv_tau) {
    const T half = c.half, gm1 = c.gm1;
    const T rho = q[0], mx = q[1], my = q[2], mz = q[3], Bx = q[4], By = q[5], Bz = q[6], e = q[7];
    const T rinv = c.one / rho;
    const T ux = mx * rinv, uy = my * rinv, uz = mz * rinv;
    const T b2 = Bx * Bx + By * By + Bz * Bz;
    const T p = (e - half * (mx * ux + my * uy + mz * uz + b2)) * gm1;
    const T ptot = p + half * b2;
    out(0, mx);
    out(1, my);
    out(2, mz);
    out(3, mx * ux - Bx * Bx + ptot);
    out(4, my * ux - By * Bx);
    out(5, mz * ux - Bz * Bx);
    out(6, mx * uy - Bx * By);
    out(7, my * uy - By * By + ptot);
    out(8, mz * uy - Bz * By);
    out(9, mx * uz - Bx * Bz);
    out(10, my * uz - By * Bz);
    out(11, mz * uz - Bz * Bz + ptot);
    T ex = uz * By - uy * Bz, ey = ux * Bz - uz * Bx, ez = uy * Bx - ux * By;
    if (hall) {
      const T dr = c.di * rinv;
      const T Jx = q[8], Jy = q[9], Jz = q[10];
      ex = ex + dr * (Jy * Bz - Jz * By);
      ey = ey + dr * (Jz * Bx - Jx * Bz);
      ez = ez + dr * (Jx * By - Jy * Bx);
    }
    out(12, ex);
    out(13, ey);
    out(14, ez);
    const T ep = e + ptot;
    const T udotb = ux * Bx + uy * By + uz * Bz;
    out(15, ep * ux - udotb * Bx);
    out(16, ep * uy - udotb * By);
    out(17, ep * uz - udotb * Bz);
    if (aeb) {
      const T two = c.two;
      out(18, c.cg * p * inv_tau - (two * Bx * Bx + By * By + Bz * Bz) * inv_tau - (mx * ux + two * my * uy + two * mz * uz) * inv_tau);
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


// rows per block and lines per FFT batch: 24 lines of 2 rows hold the 22 inputs of two rows
// (Hall) in one batch and their 38 outputs in two
template <int NX> struct PassCCfg {
  static constexpr int H = NX / 2;
  static constexpr int TPL = Plan<H>::TPL;
  static constexpr int MUL = TPL >= 4 ? 1 : 4 / TPL;
  static constexpr int LB = 24 * MUL;       // lines per batch
  static constexpr int THREADS = LB * TPL;
  static constexpr int ROWS = 2 * MUL;
  static constexpr int NF = 19;             // line slots per row
  static constexpr int LC = RowLen<H>::V;   // padded complex per line
  static constexpr int SMEM = ROWS * NF * LC * 16;
};

template <class T, int NX, int CFL>
__global__ void __launch_bounds__(PassCCfg<NX>::THREADS, 2) k_passC(Bufs<T> b, PassArgs a, PT<T> pc, const typename Store<T>::C* __restrict__ twx) {
  using CF = PassCCfg<NX>;
  using C = typename Store<T>::C;
  using SR = typename Store<T>::R;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double red[32];
  if (a.st->halt) return;
  C* sc = reinterpret_cast<C*>(smem_raw);  // [row][field] lines of LC complex
  SR* sr = reinterpret_cast<SR*>(smem_raw);
  const Geo& g = a.g;
  const int nin = a.hall ? 11 : 8;
  const int nfl = a.cfl == 2 ? 0 : (a.aeb ? 19 : 18);  // a.cfl == 2: CFL minimum only
  long long row0 = (long long)blockIdx.x * CF::ROWS;  // row = z*ny + y
  const int lt = threadIdx.x % CF::TPL, lb = threadIdx.x / CF::TPL;
  // ---- c2r of the inputs
  for (int L0 = 0; L0 < CF::ROWS * nin; L0 += CF::LB) {
    int L = L0 + lb;
    bool act = L < CF::ROWS * nin;
    int rr = act ? L / nin : 0, f = act ? L % nin : 0;
    C* z = sc + (rr * CF::NF + f) * CF::LC;
    if (act) {
      const C* xin = b.W2 + f * g.fsc + (row0 + rr) * g.kxp;
      int kk = g.kx_keep;
      c2r_pre<T, CF::H>(z, lt, [&](int k) { return k < kk ? Store<T>::ldg(xin + k) : cx_zero<T>(); }, twx);
    }
    __syncthreads();
    fft_lines<T, CF::H, +1, 1, 0>(z, 0, lt, act, twx, 2);
  }
  // ---- physics per point, in place (inputs and outputs of a point share its slots)
  T tmin = Real<T>::inf();
  bool nan_seen = false;
  const T rfac = Real<T>::from_d(a.st->radius / a.P.R0);
  const T inv_tau = Real<T>::from_d(a.st->inv_tau);
#pragma unroll 1
  for (int p = threadIdx.x; p < CF::ROWS * NX; p += CF::THREADS) {
    int rr = p / NX, xx = row_real_idx(p % NX);
    SR* base = sr + 2 * rr * CF::NF * CF::LC + xx;
    T q[11];
#pragma unroll
    for (int f = 0; f < 11; f++) q[f] = f < nin ? Store<T>::ld(base + 2 * f * CF::LC) : pc.zero;
    if (CFL) {
      T d = Flux<T>::cfl(q, pc, a.hall, rfac);
      if (Real<T>::isnan_(d)) nan_seen = true;
      else tmin = Real<T>::min_(tmin, d);
    }
    if (nfl > 0) Flux<T>::eval(q, [&](int k, T v) { Store<T>::st(base + 2 * k * CF::LC, v); }, pc, a.hall, a.aeb, inv_tau);
  }
  if (CFL) {
    double dmin = Real<T>::to_d(tmin);
    for (int o = 16; o > 0; o >>= 1) dmin = fmin(dmin, __shfl_xor_sync(0xffffffffu, dmin, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = dmin;
    if (__any_sync(0xffffffffu, nan_seen) && (threadIdx.x & 31) == 0) atomicOr(&a.st->status, LAPS_STATUS_NAN);
  }
  __syncthreads();
  if (CFL && threadIdx.x == 0) {
    double m = red[0];
    for (int w = 1; w < CF::THREADS / 32; w++) m = fmin(m, red[w]);
    atomicMin(&a.st->cfl_bits, (unsigned long long)__double_as_longlong(m));
  }
  if (nfl == 0) return;
  // ---- r2c of the fluxes
  const int sexp = -__ffs(NX) + 1;  // 1/nx
  for (int L0 = 0; L0 < CF::ROWS * nfl; L0 += CF::LB) {
    int L = L0 + lb;
    bool act = L < CF::ROWS * nfl;
    int rr = act ? L / nfl : 0, f = act ? L % nfl : 0;
    C* z = sc + (rr * CF::NF + f) * CF::LC;
    fft_lines<T, CF::H, -1, 1, 0>(z, 0, lt, act, twx, 2);
    if (act) {
      C* xo = b.W1 + f * g.fsc + (row0 + rr) * g.kxp;
      int kk = g.kx_keep;
      r2c_post<T, CF::H>(z, lt, [&](int k, cx<T> v) { if (k < kk) Store<T>::stc(xo + k, v); }, sexp, twx);
    }
  }
}

// ============================================================================ pass D
// forward y-FFT of the fluxes with the kx, ky parts of the spectral right-hand side folded
// in (calc_rhs, mhdrhs.f90:206-233), leaving only the kz parts for pass E.  Output slots:
//   0 Q1 = -(i ax F1 + i ay F2)      1 F3
//   2 Q2 = -(i ax F4 + i ay F5)      3 F6
//   4 Q3 = -(i ax F7 + i ay F8)      5 F9
//   6 Q4 = -(i ax F10 + i ay F11)    7 F12
//   8 Ex   9 Ey   10 P7 = i ay Ex - i ax Ey   11 P5 = -i ay Ez   12 P6 = i ax Ez
//   13 Q8 = -(i ax F16 + i ay F17) + Expand   14 F18
// One group per blockIdx.z (12 groups); tile: kx0..kx0+7, one z plane; reads all y of W1,
// writes kept ky rows of W2.
struct DGroup { signed char in[3], kind, out; };
enum { DG_Q = 0, DG_COPY, DG_EXY, DG_EZ, DG_Q8 };
__constant__ DGroup c_dgroups[12] = {
    {{0, 1, -1}, DG_Q, 0},  {{2, -1, -1}, DG_COPY, 1},  {{3, 4, -1}, DG_Q, 2},    {{5, -1, -1}, DG_COPY, 3},
    {{6, 7, -1}, DG_Q, 4},  {{8, -1, -1}, DG_COPY, 5},  {{9, 10, -1}, DG_Q, 6},   {{11, -1, -1}, DG_COPY, 7},
    {{12, 13, -1}, DG_EXY, 8}, {{14, -1, -1}, DG_EZ, 11}, {{15, 16, 18}, DG_Q8, 13}, {{17, -1, -1}, DG_COPY, 14}};

template <class T, int NY>
__global__ void __launch_bounds__(Col<T, NY>::THREADS) k_passD(Bufs<T> b, PassArgs a, PT<T> pc, KTab<T> K, const typename Store<T>::C* __restrict__ twy) {
  using CL = Col<T, NY>;
  using C = typename Store<T>::C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  if (a.st->halt) return;
  ColCtx<T, NY, 2> x(reinterpret_cast<C*>(smem_raw));
  const Geo& g = a.g;
  const DGroup grp = c_dgroups[blockIdx.z];
  int kx = blockIdx.x * TX + x.c;
  int z = blockIdx.y * CL::NTILE + x.tl;
  bool ok = kx < g.kx_keep && z < g.nz;
  long long col = (long long)z * g.ny * g.kxp + kx;
  T rr = Real<T>::from_d(a.st->r_ratio);
  const int sexp = -__ffs(NY) + 1;
  const int nin = grp.in[1] < 0 ? 1 : (grp.in[2] < 0 || !a.aeb ? 2 : 3);
#pragma unroll 1
  for (int k = 0; k < nin; k++) {
    const int bi = k == 0 ? 0 : 1;
    const C* in = b.W1 + grp.in[k] * g.fsc + col;
#pragma unroll 4
    for (int m = 0; m < CL::EPT; m++) {
      cx<T> v = ok ? Store<T>::ldg(in + (long long)x.j(m) * g.kxp) : cx_zero<T>();
      Store<T>::stc(x.at(bi, m), v);
    }
    __syncthreads();
    fft_lines<T, NY, -1, TX, 1>(x.buf(bi), x.c, x.t, true, twy, 1);
    if (grp.kind == DG_Q8 && k == 1) {  // fold the first two into buffer 0 before the third
#pragma unroll 2
      for (int m = 0; m < CL::EPT; m++) {
        T ax, ay, az;
        kfac(K, a.P, pc, rr, kx, x.j(m), 0, ax, ay, az);
        cx<T> q = -(mul_i(Store<T>::ldc(x.at(0, m)), ax) + mul_i(Store<T>::ldc(x.at(1, m)), ay));
        Store<T>::stc(x.at(0, m), q);
      }
      __syncthreads();
    }
  }
  if (!ok) return;
#pragma unroll 2
  for (int m = 0; m < CL::EPT; m++) {
    int ky = x.j(m);
    if (!g.ky_in(ky)) continue;
    T ax, ay, az;
    kfac(K, a.P, pc, rr, kx, ky, 0, ax, ay, az);
    cx<T> v0 = Store<T>::ldc(x.at(0, m));
    v0 = {Real<T>::mul_pow2(v0.re, sexp), Real<T>::mul_pow2(v0.im, sexp)};
    cx<T> v1 = cx_zero<T>();
    if (nin > 1) {
      v1 = Store<T>::ldc(x.at(1, m));
      v1 = {Real<T>::mul_pow2(v1.re, sexp), Real<T>::mul_pow2(v1.im, sexp)};
    }
    C* o = b.W2 + col + (long long)ky * g.kxp;
    switch (grp.kind) {
      case DG_Q: Store<T>::stc(o + grp.out * g.fsc, -(mul_i(v0, ax) + mul_i(v1, ay))); break;
      case DG_COPY: Store<T>::stc(o + grp.out * g.fsc, v0); break;
      case DG_EXY:
        Store<T>::stc(o + 8 * g.fsc, v0);
        Store<T>::stc(o + 9 * g.fsc, v1);
        Store<T>::stc(o + 10 * g.fsc, mul_i(v0, ay) - mul_i(v1, ax));
        break;
      case DG_EZ:
        Store<T>::stc(o + 11 * g.fsc, -mul_i(v0, ay));
        Store<T>::stc(o + 12 * g.fsc, mul_i(v0, ax));
        break;
      default:  // DG_Q8: buffer 0 holds the folded -(i ax F16 + i ay F17), buffer 1 the expansion term
        Store<T>::stc(o + 13 * g.fsc, nin == 3 ? v0 + v1 : v0);
        break;
    }
  }
}

// ============================================================================ pass E
// forward z-FFT with the kz parts of the right-hand side, then for variable v = blockIdx.z:
// the expansion damping (mhdrhs.f90:235-251), explicit diffusion (:253-275), the RK3 update
// with implicit diffusion (rktmod.f90:34-62) and the dealias mask or filter
// (dealiasing.f90:70-113).  Tile: kx0..kx0+7, one kept ky row; reads all z of W2, writes
// kept kz of U (and R).
template <class T, int NZ>
__global__ void __launch_bounds__(Col<T, NZ>::THREADS) k_passE(Bufs<T> b, PassArgs a, PT<T> pc, KTab<T> K, const typename Store<T>::C* __restrict__ twz) {
  using CL = Col<T, NZ>;
  using C = typename Store<T>::C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  if (a.st->halt) return;
  ColCtx<T, NZ, 2> x(reinterpret_cast<C*>(smem_raw));
  const Geo& g = a.g;
  const Phys& P = a.P;
  const int v = blockIdx.z;
  int kx = blockIdx.x * TX + x.c;
  int r = blockIdx.y * CL::NTILE + x.tl;
  bool ok = kx < g.kx_keep && r < g.nky();
  int ky = ok ? g.ky_of(r) : 0;
  long long col = (long long)ky * g.kxp + kx;
  long long zs = (long long)g.ny * g.kxp;
  const int sexp = -__ffs(NZ) + 1;
  // inputs per variable: first (plain), second (times s * i kz), s = +-1 or 0 (none)
  const int in1 = v == 4 ? 11 : v == 5 ? 12 : v == 6 ? 10 : v == 7 ? 13 : 2 * v;
  const int in2 = v == 4 ? 9 : v == 5 ? 8 : v == 6 ? -1 : v == 7 ? 14 : 2 * v + 1;
  const int nin = in2 < 0 ? 1 : 2;
#pragma unroll 1
  for (int k = 0; k < nin; k++) {
    const C* in = b.W2 + (k == 0 ? in1 : in2) * g.fsc + col;
#pragma unroll 4
    for (int m = 0; m < CL::EPT; m++) {
      cx<T> w = ok ? Store<T>::ldg(in + x.j(m) * zs) : cx_zero<T>();
      Store<T>::stc(x.at(k, m), w);
    }
    __syncthreads();
    fft_lines<T, NZ, -1, TX, 1>(x.buf(k), x.c, x.t, true, twz, 1);
  }
  if (!ok) return;
  const int stg = a.stage;
  const T cc = Real<T>::from_d(a.st->cc[stg]), ddc = Real<T>::from_d(a.st->ddc[stg]);
  const T ts = Real<T>::from_d(a.st->ts[stg]);
  const T ebmv = pc.ebm[v] * Real<T>::from_d(a.st->inv_tau);
  const T rr = Real<T>::from_d(a.st->r_ratio);
  const int plain = a.st->ksq_plain;
  const bool mom = v >= 1 && v <= 3, mag = v >= 4 && v <= 6;
  const bool need_k2 = (mom && P.visc) || (mag && P.resis);
  C* U = b.U + v * g.fsc + col;
  C* R = b.R + v * g.fsc + col;
#pragma unroll 2
  for (int m = 0; m < CL::EPT; m++) {
    int kz = x.j(m);
    if (!g.kz_in(kz)) continue;
    cx<T> fnl = Store<T>::ldc(x.at(0, m));
    fnl = {Real<T>::mul_pow2(fnl.re, sexp), Real<T>::mul_pow2(fnl.im, sexp)};
    if (nin > 1) {
      cx<T> w = Store<T>::ldc(x.at(1, m));
      w = mul_i(cx<T>{Real<T>::mul_pow2(w.re, sexp), Real<T>::mul_pow2(w.im, sexp)}, K.kzd[kz]);
      fnl = v == 4 ? fnl + w : fnl - w;
    }
    long long idx = kz * zs;
    cx<T> u = Store<T>::ldg(U + idx);
    T k2 = pc.zero;
    if (need_k2) {
      if (P.corot && !plain) k2 = ksq(K, P, pc, rr, kx, ky, kz);
      else k2 = (K.kx2[kx] + K.ky2[ky]) + K.kz2[kz];
    }
    if (P.aeb && v < 7) fnl = fnl - u * ebmv;
    if (mom && P.visc && P.visc_exp) fnl = fnl - u * (pc.nu * k2);
    if (mag && P.resis && P.resis_exp && !(P.cons_bg && kx == 0 && kz == 0)) fnl = fnl - u * (pc.eta * k2);
    cx<T> un = fnl * cc + u;
    if (stg > 0) un = (fnl * cc + Store<T>::ldg(R + idx) * ddc) + u;
    if (a.store_rk) Store<T>::stc(R + idx, fnl);
    if (mom && P.visc && !P.visc_exp) {
      T d = ts * k2 * pc.nu + pc.one;
      un = {un.re / d, un.im / d};
    }
    if (mag && P.resis && !P.resis_exp) {
      T d = ts * k2 * pc.eta + pc.one;
      un = {un.re / d, un.im / d};
    }
    if (P.dealias == 1) {
      if (kx >= K.kxlim[kz * g.ny + ky]) un = cx_zero<T>();
    } else if (P.dealias == 2) {
      un = ((un * K.fx[kx]) * K.fy[ky]) * K.fz[kz];
    }
    Store<T>::stc(U + idx, un);
  }
}

}  // namespace laps
