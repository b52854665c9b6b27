// The five fused passes of one RK stage of the 3-D compressible solver (see kernels.cuh).
//
// Column passes (A, B, D, E) spread their fields over blockIdx.z: one CTA transforms one
// tile (TX adjacent columns) of one field group, so each CTA runs 1-3 FFTs and keeps
// partial results in shared-memory buffers, not registers.
#pragma once
#include <type_traits>
#include "kernels.cuh"
#include "tma.cuh"

namespace laps {

struct PassArgs {
  Geo g;
  Phys P;
  int hall, aeb;
  int stage;       // 0, 1, 2
  int store_rk;    // write fnl_rk (not needed after the last stage of a fused step)
  int cfl;         // pass C: 0 fluxes, 1 fluxes + CFL minimum, 2 CFL minimum only
  int mass_from_state;  // compressible, Nyquist modes zeroed by the dealiasing: the mass
                        // flux rho u is the state's momentum, so -i k.(rho u)^ is taken from U
                        // in pass E and passes C, D skip fluxes 1..3
  int e_first;     // pass E: variable of blockIdx.z = 0 (the continuity update runs in a launch
                   // of its own before the momentum is overwritten)
  int rhs_only;    // store the right-hand side (fnl) in R and leave the state (laps_calc_rhs)
  int mass_done;   // the continuity update (k_mass_rk) was launched already, beside pass D
  int sched;       // execution schedule bits (LAPS_SCHED_*): results do not depend on them
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
// inverse z-FFT of output f = blockIdx.z: state field src[f], optionally times -i kz or +i kz:
//   compressible:   0..7 state, 8: C_x = IFFT_z(-i kz B_y), 9: C_y = IFFT_z(i kz B_x) (Hall)
//   incompressible: 0..6 state, 7: C_x, 8: C_y, 9..11: IFFT_z(i kz (rho u)_c), c = x, y, z
// Tile: kx0..kx0+7, one kept ky row; writes all z of W1.  (Not used in 2-D: nz = 1.)
struct ATab { signed char src, mult; };
__constant__ ATab c_atab[2][12] = {
    {{0, 0}, {1, 0}, {2, 0}, {3, 0}, {4, 0}, {5, 0}, {6, 0}, {7, 0}, {5, -1}, {4, 1}, {0, 0}, {0, 0}},
    {{0, 0}, {1, 0}, {2, 0}, {3, 0}, {4, 0}, {5, 0}, {6, 0}, {5, -1}, {4, 1}, {1, 1}, {2, 1}, {3, 1}}};

template <class T, class TS, int NZ>
__global__ void __launch_bounds__(Col<T, NZ>::THREADS)
    k_passA(Bufs<T, TS> b, PassArgs a, PassK<T, TS> kk, const typename Store<T>::C* __restrict__ twz,
            const __grid_constant__ CUtensorMap tmap) {
  const PT<T>& pc = kk.pc;
  const KTab<T>& K = kk.K;
  using CL = Col<T, NZ>;
  using C = typename Store<T>::C;
  using CS = typename Store<TS>::C;
  extern __shared__ __align__(128) unsigned char smem_tma[];  // 128-byte aligned: TMA destinations
  __shared__ __align__(8) uint64_t tbar[2];
  if (a.st->halt) return;
  ColCtx<T, NZ, 1> x(reinterpret_cast<C*>(smem_tma));
  // the state tiles (whole z columns, state type) share the block's shared memory with the
  // transform tiles: every thread takes its elements from them into registers before the
  // first transform element is written (the state type is at least as wide as the compute type)
  static_assert(sizeof(CS) >= sizeof(C), "state tiles cover the transform tiles");
  CS* raw = reinterpret_cast<CS*>(smem_tma) + x.tl * NZ * TX;
  const Geo& g = a.g;
  const int f = blockIdx.z;
  const ATab e = c_atab[a.P.variant == LAPS_VARIANT_3DI ? 1 : 0][f];
  int kx = blockIdx.x * TX + x.c;
  int r = blockIdx.y * CL::NTILE + x.tl;
  bool ok = kx < g.kx_keep && r < g.nky();
  int ky = ok ? g.ky_of(r) : 0;
  long long col = (long long)ky * g.kxp + kx;  // + z * ny * kxp
  long long zs = (long long)g.ny * g.kxp;
  {
    TileLoad tl;
    tl.init(tbar);
    if (threadIdx.x == 0) {
      // only the kept kz rows of each column (the map's box is kc.box rows high)
      constexpr int EW = (int)(sizeof(CS) / 8);
      const KeptCopies kc(g.kz_lo, g.kz_hi, NZ, tile_gran((int)sizeof(CS)));
      const int nc = kc.count(NZ);
      const int r0 = blockIdx.y * CL::NTILE;
      const int nt = g.nky() - r0 < CL::NTILE ? g.nky() - r0 : CL::NTILE;
      tl.expect(0, (uint32_t)(nt * nc * kc.box * TX * (int)sizeof(CS)));
      for (int t = 0; t < nt; t++) {
        CS* dst = reinterpret_cast<CS*>(smem_tma) + t * NZ * TX;
        for (int i = 0; i < nc; i++) {
          const int z0 = kc.start(i, NZ);
          tl.copy(0, dst + z0 * TX, &tmap, blockIdx.x * TX * EW, g.ky_of(r0 + t), e.src * g.nz + z0);
        }
      }
    }
    if (!tl.wait(0, a.st)) return;
  }
  cx<T> v[CL::EPT];
#pragma unroll
  for (int m = 0; m < CL::EPT; m++) {
    int kz = x.j(m);
    v[m] = cx_zero<T>();
    if (ok && g.kz_in(kz)) {
      // (FP32 lines of an FP64 state: the conversion on the integer pipes)
      if constexpr (std::is_same<T, float>::value) v[m] = IncCvt<TS>::to_f32(Store<TS>::ldc(raw + kz * TX + x.c));
      else v[m] = cvtc<T>(Store<TS>::ldc(raw + kz * TX + x.c));
      if (e.mult < 0) v[m] = -mul_i(v[m], K.kzd[kz]);
      else if (e.mult > 0) v[m] = mul_i(v[m], K.kzd[kz]);
    }
  }
  // same element sizes: each thread rewrites only the slots it has read; narrower transform
  // elements overwrite other threads' state elements, so all reads come first
  if constexpr (sizeof(CS) != sizeof(C)) __syncthreads();
#pragma unroll
  for (int m = 0; m < CL::EPT; m++) Store<T>::stc(x.at(0, m), v[m]);
  __syncthreads();
  fft_lines<T, NZ, +1, TX, 1>(x.buf(0), x.c, x.t, true, twz, 1);
  if (!ok) return;
  C* out = b.W1 + f * g.fsc + col;
#pragma unroll
  for (int m = 0; m < CL::EPT; m++) Store<T>::stc(out + x.j(m) * zs, Store<T>::ldc(x.at(0, m)));
}

// ============================================================================ pass B
// inverse y-FFT of output f = blockIdx.z, the sum of up to two input columns each times
// 1, i ax or i ay (signed):
//   compressible 3-D: 0..7 state; J: 8 = i ay W1[Bz] + W1[Cx], 9 = W1[Cy] - i ax W1[Bz],
//                     10 = i ax W1[By] - i ay W1[Bx]
//   compressible 2-D: the same reading the state U directly (nz = 1, kz = 0: no C terms)
//   incompressible:   0..6 state; J: 7, 8, 9; grad(rho u): 10 + 3c + d = d/dx_d (rho u)_c
// Tile: kx0..kx0+7, one z plane; reads kept ky rows, writes all y of W2.
enum { BF_ONE = 1, BF_AX = 2, BF_MAX = -2, BF_AY = 3, BF_MAY = -3 };
// one tile buffer per block in 3-D pass B: FP32 lines in single-tile blocks
#ifndef LAPS_PASSB_ONEBUF
#define LAPS_PASSB_ONEBUF 1
#endif
template <class T, int N> struct PassBOneBuf {
  static constexpr bool V = LAPS_PASSB_ONEBUF && sizeof(typename Store<T>::C) == 8 && Col<T, N>::NTILE == 1;
};
struct BTab { signed char in0, f0, in1, f1; };
__constant__ BTab c_btab[3][19] = {
    {{0, 1, -1, 0}, {1, 1, -1, 0}, {2, 1, -1, 0}, {3, 1, -1, 0}, {4, 1, -1, 0}, {5, 1, -1, 0}, {6, 1, -1, 0}, {7, 1, -1, 0},
     {6, BF_AY, 8, BF_ONE}, {9, BF_ONE, 6, BF_MAX}, {5, BF_AX, 4, BF_MAY}},
    {{0, 1, -1, 0}, {1, 1, -1, 0}, {2, 1, -1, 0}, {3, 1, -1, 0}, {4, 1, -1, 0}, {5, 1, -1, 0}, {6, 1, -1, 0}, {7, 1, -1, 0},
     {6, BF_AY, -1, 0}, {6, BF_MAX, -1, 0}, {5, BF_AX, 4, BF_MAY}},
    {{0, 1, -1, 0}, {1, 1, -1, 0}, {2, 1, -1, 0}, {3, 1, -1, 0}, {4, 1, -1, 0}, {5, 1, -1, 0}, {6, 1, -1, 0},
     {6, BF_AY, 7, BF_ONE}, {8, BF_ONE, 6, BF_MAX}, {5, BF_AX, 4, BF_MAY},
     {1, BF_AX, -1, 0}, {1, BF_AY, -1, 0}, {9, BF_ONE, -1, 0},
     {2, BF_AX, -1, 0}, {2, BF_AY, -1, 0}, {10, BF_ONE, -1, 0},
     {3, BF_AX, -1, 0}, {3, BF_AY, -1, 0}, {11, BF_ONE, -1, 0}}};

template <class T>
__device__ __forceinline__ cx<T> bterm(cx<T> v, int f, T ax, T ay) {
  switch (f) {
    case BF_AX: return mul_i(v, ax);
    case BF_MAX: return -mul_i(v, ax);
    case BF_AY: return mul_i(v, ay);
    case BF_MAY: return -mul_i(v, ay);
    default: return v;
  }
}

template <class T, class TS, int NY>
__global__ void __launch_bounds__(Col<T, NY>::THREADS)
    k_passB(Bufs<T, TS> b, PassArgs a, PassK<T, TS> kk, const typename Store<T>::C* __restrict__ twy,
            const __grid_constant__ CUtensorMap tmap) {
  const PT<T>& pc = kk.pc;
  const KTab<T>& K = kk.K;
  using CL = Col<T, NY>;
  using C = typename Store<T>::C;
  extern __shared__ __align__(128) unsigned char smem_tma[];  // 128-byte aligned: TMA destinations
  __shared__ __align__(8) uint64_t tbar[2];
  if (a.st->halt) return;
  ColCtx<T, NY, 2> x(reinterpret_cast<C*>(smem_tma));
  const Geo& g = a.g;
  const int f = blockIdx.z;
  const int vt = a.P.variant == LAPS_VARIANT_3DI ? 2 : (a.P.two_d ? 1 : 0);
  const BTab e = c_btab[vt][f];
  const bool from_state = a.P.two_d;
  int kx = blockIdx.x * TX + x.c;
  int z = blockIdx.y * CL::NTILE + x.tl;
  bool ok = kx < g.kx_keep && z < g.nz;
  long long col = (long long)z * g.ny * g.kxp + kx;  // + y * kxp
  T rr = Real<T>::from_d(a.st->r_ratio);
  const bool kf = e.f0 > 1 || e.f0 < 0 || e.f1 > 1 || e.f1 < 0;
  if (!from_state) {
    // 3-D: the input tiles (whole y columns) come by TMA into buffers 0 and 1, then each
    // thread forms its elements of the output in buffer 0 (zero outside the kept ky rows)
    TileLoad tl;
    tl.init(tbar);
    const int nin = e.in1 >= 0 ? 2 : 1;
    // FP32 single-tile blocks hold one buffer: a second input comes into it once the threads
    // have taken the first into registers (twice the resident blocks of two buffers)
    constexpr bool SEQ = PassBOneBuf<T, NY>::V;
    // only the kept ky rows of each column (the map's box is kc.box rows high); input k into
    // buffer `buf` of every tile, announced on barrier k
    auto issue = [&](int k, int buf) {
      if (threadIdx.x != 0) return;
      constexpr int EW = (int)(sizeof(C) / 8);
      const KeptCopies kc(g.ky_lo, g.ky_hi, NY, tile_gran((int)sizeof(C)));
      const int nc = kc.count(NY);
      const int z0 = blockIdx.y * CL::NTILE;
      const int nt = g.nz - z0 < CL::NTILE ? g.nz - z0 : CL::NTILE;
      tl.expect(k, (uint32_t)(nt * nc * kc.box * TX * (int)sizeof(C)));
      for (int t = 0; t < nt; t++) {
        C* dst = reinterpret_cast<C*>(smem_tma) + (t * 2 + buf) * NY * TX;  // tile t, buffer buf
        for (int i = 0; i < nc; i++) {
          const int y0 = kc.start(i, NY);
          tl.copy(k, dst + y0 * TX, &tmap, blockIdx.x * TX * EW, y0, (k == 0 ? e.in0 : e.in1) * g.nz + z0 + t);
        }
      }
    };
    if constexpr (SEQ) {
      issue(0, 0);
      if (!tl.wait(0, a.st)) return;
      cx<T> v[CL::EPT];
#pragma unroll
      for (int m = 0; m < CL::EPT; m++) {
        const int ky = x.j(m);
        v[m] = cx_zero<T>();
        if (ok && g.ky_in(ky)) {
          T ax = pc.zero, ay = pc.zero, az;
          if (kf) kfac(K, a.P, pc, rr, kx, ky, 0, ax, ay, az);
          v[m] = bterm(Store<T>::ldc(x.at(0, m)), e.f0, ax, ay);
        }
      }
      if (nin > 1) {
        __syncthreads();  // every thread has read the first input
        if (threadIdx.x == 0) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        issue(1, 0);
        if (!tl.wait(1, a.st)) return;
#pragma unroll
        for (int m = 0; m < CL::EPT; m++) {
          const int ky = x.j(m);
          if (ok && g.ky_in(ky)) {
            T ax = pc.zero, ay = pc.zero, az;
            if (kf) kfac(K, a.P, pc, rr, kx, ky, 0, ax, ay, az);
            v[m] = v[m] + bterm(Store<T>::ldc(x.at(0, m)), e.f1, ax, ay);
          }
        }
      }
#pragma unroll
      for (int m = 0; m < CL::EPT; m++) Store<T>::stc(x.at(0, m), v[m]);
    } else {
    issue(0, 0);
    if (nin > 1) issue(1, 1);
    if (!tl.wait(0, a.st) || (nin > 1 && !tl.wait(1, a.st))) return;
#pragma unroll
    for (int m = 0; m < CL::EPT; m++) {
      int ky = x.j(m);
      cx<T> v = cx_zero<T>();
      if (ok && g.ky_in(ky)) {
        T ax = pc.zero, ay = pc.zero, az;
        if (kf) kfac(K, a.P, pc, rr, kx, ky, 0, ax, ay, az);
        v = bterm(Store<T>::ldc(x.at(0, m)), e.f0, ax, ay);
        if (nin > 1) v = v + bterm(Store<T>::ldc(x.at(1, m)), e.f1, ax, ay);
      }
      Store<T>::stc(x.at(0, m), v);
    }
    }
  } else {
    // 2-D: the state itself (the state type) through the threads
#pragma unroll
    for (int m = 0; m < CL::EPT; m++) {
      int ky = x.j(m);
      cx<T> v = cx_zero<T>();
      if (ok && g.ky_in(ky)) {
        const long long off = col + (long long)ky * g.kxp;
        auto ld = [&](int fi) { return cvtc<T>(Store<TS>::ldg(b.U + off + fi * g.fsc)); };
        T ax = pc.zero, ay = pc.zero, az;
        if (kf) kfac(K, a.P, pc, rr, kx, ky, 0, ax, ay, az);
        v = bterm(ld(e.in0), e.f0, ax, ay);
        if (e.in1 >= 0) v = v + bterm(ld(e.in1), e.f1, ax, ay);
      }
      Store<T>::stc(x.at(0, m), v);
    }
  }
  __syncthreads();
  fft_lines<T, NY, +1, TX, 1>(x.buf(0), x.c, x.t, true, twy, 1);
  if (!ok) return;
  C* out = b.W2 + f * g.fsc + col;
#pragma unroll
  for (int m = 0; m < CL::EPT; m++) Store<T>::stc(out + (long long)x.j(m) * g.kxp, Store<T>::ldc(x.at(0, m)));
}

// Pass B for FP32 lines of a 3-D run, persistent and double-buffered: each block takes items
// (kx tile, z tile, output f) in turn, and the TMA loads of its next item go out before the
// current item is combined, transformed and stored, so that the loads' latency overlaps the
// block's own work instead of leaving it idle between one-shot launches.  Two buffer sets of
// two buffers per tile (ColCtx with 4 buffers), one mbarrier per buffer, reused every other
// item with its phase parity kept in a register.
template <class T, class TS, int NY>
__global__ void __launch_bounds__(Col<T, NY>::THREADS)
    k_passB_pipe(Bufs<T, TS> b, PassArgs a, PassK<T, TS> kk, const typename Store<T>::C* __restrict__ twy,
                 const __grid_constant__ CUtensorMap tmap, int nitems, int nbx, int nby) {
  const PT<T>& pc = kk.pc;
  const KTab<T>& K = kk.K;
  using CL = Col<T, NY>;
  using C = typename Store<T>::C;
  extern __shared__ __align__(128) unsigned char smem_tma[];
  __shared__ __align__(8) uint64_t tbar[4];
  if (a.st->halt) return;
  ColCtx<T, NY, 4> x(reinterpret_cast<C*>(smem_tma));
  const Geo& g = a.g;
  const int vt = a.P.variant == LAPS_VARIANT_3DI ? 2 : 0;
  const T rr = Real<T>::from_d(a.st->r_ratio);
  // barrier 2 set + k holds buffer k of a set; bit i of ph is the parity barrier i waits on next
  uint32_t ph = 0;
  if (threadIdx.x == 0) {
    for (int i = 0; i < 4; i++) mbar_init(&tbar[i], 1);
    mbar_fence_init();
  }
  __syncthreads();
  auto wait_buf = [&](int i) -> bool {  // every thread; false (after reporting) when the wait ran out
    const bool good = mbar_wait(&tbar[i], (ph >> i) & 1u);
    ph ^= 1u << i;
    if (!good) atomicOr(&a.st->status, LAPS_STATUS_DEVICE_TIMEOUT);
    return __syncthreads_and(good) != 0;
  };
  // the loads of item `it` into buffer set `set` (thread 0)
  auto issue = [&](int set, int it) {
    if (threadIdx.x != 0) return;
    const int bx = it % nbx, by = (it / nbx) % nby, f = it / (nbx * nby);
    const BTab e = c_btab[vt][f];
    const int nin = e.in1 >= 0 ? 2 : 1;
    constexpr int EW = (int)(sizeof(C) / 8);
    const KeptCopies kc(g.ky_lo, g.ky_hi, NY, tile_gran((int)sizeof(C)));
    const int nc = kc.count(NY);
    const int z0 = by * CL::NTILE;
    const int nt = g.nz - z0 < CL::NTILE ? g.nz - z0 : CL::NTILE;
    for (int k = 0; k < nin; k++) {
      uint64_t* bar = &tbar[set * 2 + k];
      mbar_arrive_expect_tx(bar, (uint32_t)(nt * nc * kc.box * TX * (int)sizeof(C)));
      for (int t = 0; t < nt; t++) {
        C* dst = reinterpret_cast<C*>(smem_tma) + (t * 4 + set * 2 + k) * NY * TX;  // tile t, set, buffer k
        for (int i = 0; i < nc; i++) {
          const int y0 = kc.start(i, NY);
          tma_load_3d(dst + y0 * TX, &tmap, bx * TX * EW, y0, (k == 0 ? e.in0 : e.in1) * g.nz + z0 + t, bar);
        }
      }
    }
  };
  int it = blockIdx.x;
  if (it >= nitems) return;
  issue(0, it);
#pragma unroll 1
  for (int set = 0; it < nitems; it += gridDim.x, set ^= 1) {
    const int nxt = it + gridDim.x;
    if (nxt < nitems) {
      // the other set was last read in the previous item, which ended on a block barrier
      if (threadIdx.x == 0) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      issue(set ^ 1, nxt);
    }
    const int bx = it % nbx, by = (it / nbx) % nby, f = it / (nbx * nby);
    const BTab e = c_btab[vt][f];
    const int nin = e.in1 >= 0 ? 2 : 1;
    const int kx = bx * TX + x.c, z = by * CL::NTILE + x.tl;
    const bool ok = kx < g.kx_keep && z < g.nz;
    const long long col = (long long)z * g.ny * g.kxp + kx;
    const bool kf = e.f0 > 1 || e.f0 < 0 || e.f1 > 1 || e.f1 < 0;
    if (!wait_buf(set * 2) || (nin > 1 && !wait_buf(set * 2 + 1))) return;
    C* b0 = x.buf(set * 2);
#pragma unroll
    for (int m = 0; m < CL::EPT; m++) {
      const int ky = x.j(m);
      cx<T> v = cx_zero<T>();
      if (ok && g.ky_in(ky)) {
        T ax = pc.zero, ay = pc.zero, az;
        if (kf) kfac(K, a.P, pc, rr, kx, ky, 0, ax, ay, az);
        v = bterm(Store<T>::ldc(x.at(set * 2, m)), e.f0, ax, ay);
        if (nin > 1) v = v + bterm(Store<T>::ldc(x.at(set * 2 + 1, m)), e.f1, ax, ay);
      }
      Store<T>::stc(x.at(set * 2, m), v);
    }
    __syncthreads();
    fft_lines<T, NY, +1, TX, 1>(b0, x.c, x.t, true, twy, 1);
    if (ok) {
      C* out = b.W2 + f * g.fsc + col;
#pragma unroll
      for (int m = 0; m < CL::EPT; m++) Store<T>::stc(out + (long long)x.j(m) * g.kxp, Store<T>::ldc(x.at(set * 2, m)));
    }
    __syncthreads();
  }
}

// ============================================================================ pass C
// Per x-row (y, z): c2r of the inputs, the real-space physics, the CFL minimum of vardt when
// asked, and r2c of the outputs.
//   compressible (Flux): calc_flux (mhdrhs.f90:21-124, 2D/mhdrhs.f90:23-132) with the
//     primitives of update_uu_prim_from_uu (:282-294); 11 inputs (8 state + J), 18 (+1) outputs
//   incompressible (FluxI): calc_flux_for_pressure and calc_flux
//     (src_incompressible/mhdrhs.f90:25-84,393-437); 19 inputs (7 state, J, grad(rho u)),
//     6 outputs (pressure flux, E)
template <class T>
struct Flux {
  // in: rho, mx, my, mz, Bx, By, Bz, e, Jx, Jy, Jz ; out(k, value) receives the 18 fluxes and
  // the expansion term (k = 18) one at a time, so that they need not all be live at once
  template <class OUT>
  __device__ __forceinline__ static void eval(const T* q, OUT out, const PT<T>& c, const Phys& P, T inv_tau, T inv_rho0) {
    const T half = c.half, gm1 = c.gm1;
    const T rho = q[0], mx = q[1], my = q[2], mz = q[3], Bx = q[4], By = q[5], Bz = q[6], e = q[7];
    const T rinv = Real<T>::recip(rho);
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
    if (P.hall) {
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
    if (P.aeb) {
      const T two = c.two;
      if (P.zrad)  // 2D/mhdrhs.f90:96-100
        out(18, c.cg * p * inv_tau - (Bx * Bx + By * By + two * Bz * Bz) * inv_tau - (two * mx * ux + two * my * uy + mz * uz) * inv_tau);
      else
        out(18, c.cg * p * inv_tau - (two * Bx * Bx + By * By + Bz * Bz) * inv_tau - (mx * ux + two * my * uy + two * mz * uz) * inv_tau);
    }
  }
  // min over the axes of dx_i / c_max,i (mhd.f90:355-409; 2-D: x and y only, the
  // explicit-resistivity term and radial x, 2D/mhd.f90:313-392)
  template <class M = MathExact<T>>
  __device__ __forceinline__ static T cfl(const T* q, const PT<T>& c, const Phys& P, T rfac) {
    const T zero = c.zero, four = c.four, half = c.half;
    const T is2 = c.is2;
    T rho = q[0], rinv = M::div(c.one, rho);
    T ux = q[1] * rinv, uy = q[2] * rinv, uz = q[3] * rinv;
    T Bx = q[4], By = q[5], Bz = q[6];
    T p = (q[7] - half * (q[1] * ux + q[2] * uy + q[3] * uz + Bx * Bx + By * By + Bz * Bz)) * c.gm1;
    T cs2 = c.gamma * p * rinv;
    T sq = M::sqrt(rho);
    T ca[3] = {M::div(Bx, sq), M::div(By, sq), M::div(Bz, sq)};
    T u[3] = {ux, uy, uz};
    T ca2 = ca[0] * ca[0] + ca[1] * ca[1] + ca[2] * ca[2];
    T cms2 = cs2 + ca2;
    T cmax[3];
    const int nd = P.two_d ? 2 : 3;
#pragma unroll
    for (int d = 0; d < 3; d++) {
      if (d >= nd) { cmax[d] = c.one; continue; }
      T cns = M::sqrt(Real<T>::max_(cms2 * cms2 - (four * cs2) * (ca[d] * ca[d]), zero));
      T cf = M::sqrt(cms2 + cns) * is2;
      T cs = M::sqrt(Real<T>::max_(cms2 - cns, zero)) * is2;
      T m = Real<T>::abs_(u[d] + cf);
      m = Real<T>::max_(m, Real<T>::abs_(u[d] + cs));
      m = Real<T>::max_(m, Real<T>::abs_(u[d] + ca[d]));
      m = Real<T>::max_(m, Real<T>::abs_(u[d] - cf));
      m = Real<T>::max_(m, Real<T>::abs_(u[d] - cs));
      m = Real<T>::max_(m, Real<T>::abs_(u[d] - ca[d]));
      m = Real<T>::max_(m, Real<T>::abs_(u[d]));
      cmax[d] = m;
    }
    if (P.two_d && P.resis && P.resis_exp) {
      cmax[0] = Real<T>::max_(cmax[0], c.eta_dx);
      cmax[1] = Real<T>::max_(cmax[1], c.eta_dy);
    }
    if (P.hall) {
      T bm = Real<T>::max_(Real<T>::max_(Bx, By), Bz);
      T ch = c.di * rinv * bm * c.inv_mindx;
#pragma unroll
      for (int d = 0; d < 3; d++) cmax[d] = Real<T>::max_(cmax[d], ch);
    }
    T dtx = M::div(c.dx, cmax[0]);
    if (P.zrad) dtx = dtx * rfac;
    T dty = M::div(c.dy, cmax[1]) * rfac;
    if (P.two_d) return Real<T>::min_(dtx, dty);
    T dtz = M::div(c.dz, cmax[2]) * rfac;
    return Real<T>::min_(Real<T>::min_(dtx, dty), dtz);
  }
  // The FP32 screen of the CFL bound: the same speeds, with the maximum over
  // |u +- c_f|, |u +- c_s|, |u +- c_A,d|, |u| written as |u| + c_f (c_f >= c_s and
  // c_f >= |c_A,d|, so the two agree up to rounding); approximate divide and square root.
  __device__ __forceinline__ static float cfl_screen(const float* q, const PT<float>& c, const Phys& P, float rfac) {
    using M = MathFastF;
    const float rho = q[0], rinv = M::div(1.f, rho);
    const float ux = q[1] * rinv, uy = q[2] * rinv, uz = q[3] * rinv;
    const float Bx = q[4], By = q[5], Bz = q[6];
    const float p = (q[7] - 0.5f * (q[1] * ux + q[2] * uy + q[3] * uz + Bx * Bx + By * By + Bz * Bz)) * c.gm1;
    const float cs2 = c.gamma * p * rinv;
    const float b2r = (Bx * Bx + By * By + Bz * Bz) * rinv;  // c_A^2
    const float cms2 = cs2 + b2r;
    const float u[3] = {ux, uy, uz};
    const float ca2[3] = {Bx * Bx * rinv, By * By * rinv, Bz * Bz * rinv};
    float cmax[3];
    const int nd = P.two_d ? 2 : 3;
#pragma unroll
    for (int d = 0; d < 3; d++) {
      if (d >= nd) { cmax[d] = 1.f; continue; }
      const float cns = M::sqrt(fmaxf(cms2 * cms2 - 4.f * cs2 * ca2[d], 0.f));
      cmax[d] = fabsf(u[d]) + M::sqrt(0.5f * (cms2 + cns));
    }
    if (P.two_d && P.resis && P.resis_exp) {
      cmax[0] = fmaxf(cmax[0], c.eta_dx);
      cmax[1] = fmaxf(cmax[1], c.eta_dy);
    }
    if (P.hall) {
      const float ch = c.di * rinv * fmaxf(fmaxf(Bx, By), Bz) * c.inv_mindx;
#pragma unroll
      for (int d = 0; d < 3; d++) cmax[d] = fmaxf(cmax[d], ch);
    }
    float dtx = M::div(c.dx, cmax[0]);
    if (P.zrad) dtx = dtx * rfac;
    const float dty = M::div(c.dy, cmax[1]) * rfac;
    if (P.two_d) return fminf(dtx, dty);
    return fminf(fminf(dtx, dty), M::div(c.dz, cmax[2]) * rfac);
  }
};


template <class T>
struct FluxI {
  // in: rho, mx, my, mz, Bx, By, Bz, Jx, Jy, Jz, then d/dx_d (rho u)_c at 10 + 3c + d
  // (times 1/rho0 here); out: pressure flux fp (0..2) and the electric field (3..5)
  template <class OUT>
  __device__ __forceinline__ static void eval(const T* q, OUT out, const PT<T>& c, const Phys& P, T inv_tau, T inv_rho0) {
    const T rho = q[0], mx = q[1], my = q[2], mz = q[3], Bx = q[4], By = q[5], Bz = q[6];
    const T Jx = q[7], Jy = q[8], Jz = q[9];
    T g[9];
#pragma unroll
    for (int i = 0; i < 9; i++) g[i] = q[10 + i] * inv_rho0;
    out(0, -mx * g[0] - my * g[1] - mz * g[2] + Jy * Bz - Jz * By);
    out(1, -mx * g[3] - my * g[4] - mz * g[5] + Jz * Bx - Jx * Bz);
    out(2, -mx * g[6] - my * g[7] - mz * g[8] + Jx * By - Jy * Bx);
    const T rinv = Real<T>::recip(rho);
    const T ux = mx * rinv, uy = my * rinv, uz = mz * rinv;
    T ex = uz * By - uy * Bz, ey = ux * Bz - uz * Bx, ez = uy * Bx - ux * By;
    if (P.hall) {
      const T dr = c.di * rinv;
      ex = ex + dr * (Jy * Bz - Jz * By);
      ey = ey + dr * (Jz * Bx - Jx * Bz);
      ez = ez + dr * (Jx * By - Jy * Bx);
    }
    out(3, ex);
    out(4, ey);
    out(5, ez);
  }
  // Alfven-only CFL (src_incompressible/mhd.f90:394-463)
  template <class M = MathExact<T>>
  __device__ __forceinline__ static T cfl(const T* q, const PT<T>& c, const Phys& P, T rfac) {
    T rho = q[0], rinv = M::div(c.one, rho);
    T u[3] = {q[1] * rinv, q[2] * rinv, q[3] * rinv};
    T sq = M::sqrt(rho);
    T cmax[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
      T ca = M::div(q[4 + d], sq);
      T m = Real<T>::abs_(u[d] + ca);
      m = Real<T>::max_(m, Real<T>::abs_(u[d] - ca));
      m = Real<T>::max_(m, Real<T>::abs_(u[d]));
      cmax[d] = m;
    }
    if (P.hall) {
      T bm = Real<T>::max_(Real<T>::max_(q[4], q[5]), q[6]);
      T ch = c.di * rinv * bm * c.inv_mindx;
#pragma unroll
      for (int d = 0; d < 3; d++) cmax[d] = Real<T>::max_(cmax[d], ch);
    }
    T dtx = M::div(c.dx, cmax[0]);
    T dty = M::div(c.dy, cmax[1]) * rfac;
    T dtz = M::div(c.dz, cmax[2]) * rfac;
    return Real<T>::min_(Real<T>::min_(dtx, dty), dtz);
  }
  // FP32 screen: max(|u +- c_A,d|, |u|) = |u| + |c_A,d|; approximate divide and square root
  __device__ __forceinline__ static float cfl_screen(const float* q, const PT<float>& c, const Phys& P, float rfac) {
    using M = MathFastF;
    const float rho = q[0], rinv = M::div(1.f, rho), sq = M::sqrt(rho);
    float cmax[3];
#pragma unroll
    for (int d = 0; d < 3; d++) cmax[d] = fabsf(q[1 + d] * rinv) + fabsf(M::div(q[4 + d], sq));
    if (P.hall) {
      const float ch = c.di * rinv * fmaxf(fmaxf(q[4], q[5]), q[6]) * c.inv_mindx;
#pragma unroll
      for (int d = 0; d < 3; d++) cmax[d] = fmaxf(cmax[d], ch);
    }
    return fminf(fminf(M::div(c.dx, cmax[0]), M::div(c.dy, cmax[1]) * rfac), M::div(c.dz, cmax[2]) * rfac);
  }
};

// pass C transform lists (flux slot numbers): compressible, compressible with the continuity
// term from the state, incompressible; the expansion term 18 is last and dropped without it
__constant__ int c_flist[3][16] = {{0, 1, 2, 3, 4, 5, 7, 8, 11, 12, 13, 14, 15, 16, 17, 18},
                                   {3, 4, 5, 7, 8, 11, 12, 13, 14, 15, 16, 17, 18, 0, 0, 0},
                                   {0, 1, 2, 3, 4, 5, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0}};
// slots the physics has to store (all but 6, 9, 10; in the incompressible case all of 0..5)
constexpr unsigned c_fused = 0x7FFFFu & ~((1u << 6) | (1u << 9) | (1u << 10));

// Rows per block and lines per FFT batch: 24 lines of 2 rows hold the 22 inputs of two rows
// (Hall) in one batch; when two rows of 19 line slots do not fit in shared memory (1024-point
// rows of 16-byte elements) a block takes one row and batches of 12 lines.
// Lines per batch of the 512-point rows: 16 (256 threads) leaves 128 or more registers per
// thread (24 spilled: 3-D incompressible 512^3 pass C 22.7 -> 18.3 ms per step);
// LAPS_PASSC_LB_LONG overrides it at build time for tuning sweeps.
#ifndef LAPS_PASSC_LB_LONG
#define LAPS_PASSC_LB_LONG 16
#endif
// 1024-point rows of FP32 lines: one half-length complex line per row (a warp per line, no
// block barriers inside a transform) in batches of 32 lines (1024 threads): the 2-D ensemble's
// 1024^2 members, pass C -4 % against paired rows in batches of 16 (LAPS_PASSC_PAIR_1024,
// LAPS_PASSC_LB_1024 override it at build time)
#ifndef LAPS_PASSC_LB_1024
#define LAPS_PASSC_LB_1024 32
#endif
#ifndef LAPS_PASSC_PAIR_1024
#define LAPS_PASSC_PAIR_1024 0
#endif
// resident blocks of FP32 pass C the register budget is set for: 5 (64 registers, 30 warps per
// SM) measured 2 % faster at 256^3 than 4 (80 registers); the build-time override is for sweeps
#ifndef LAPS_PASSC_OCC_F32
#define LAPS_PASSC_OCC_F32 5
#endif
template <int NX, int CB> struct PassCCfg {
  static constexpr int H = NX / 2;
  static constexpr int TPL = Plan<H>::TPL;
  static constexpr int MUL = TPL >= 4 ? 1 : 4 / TPL;
  static constexpr int NF = 19;             // line slots per row
  static constexpr int LC = RowLen<H>::V;   // padded complex per line
  static constexpr bool ONE_ROW = 2 * MUL * NF * LC * CB > 200 * 1024;
  static constexpr int LB = ONE_ROW ? 12 : (NX >= 1024 ? LAPS_PASSC_LB_1024 : NX >= 512 ? LAPS_PASSC_LB_LONG : 24 * MUL);  // lines per batch
  static constexpr int THREADS = LB * TPL;
  static constexpr int ROWS = ONE_ROW ? 1 : 2 * MUL;
  // Paired rows: rows 2p and 2p+1 of a field share one complex line of NX points,
  // z = x_2p + i x_2p+1, so a row pair takes one full-length complex FFT and no twiddled
  // packing (up to 512 points; 1024-point lines would take two warps and block barriers, so
  // 1024-point rows keep the half-length form unless LAPS_PASSC_PAIR_1024 is set).
  static constexpr int TPLP = Plan<NX>::TPL;
  static constexpr bool PAIRED = !ONE_ROW && TPLP <= 64 && (NX != 1024 || LAPS_PASSC_PAIR_1024);
  static constexpr bool LWARP = TPLP <= 32;  // a paired line within one warp (else two: block barriers)
  static constexpr int LCP = RowLen<NX>::V;   // padded complex per paired line
  static constexpr int LBP = THREADS / TPLP;  // paired lines per batch
  static constexpr int FSTR = PAIRED ? 2 * LCP : 2 * LC;  // field stride in reals
  static constexpr int SMEM = (PAIRED ? (ROWS / 2) * NF * LCP : ROWS * NF * LC) * CB;  // CB: bytes of one complex
  // resident blocks per SM the register budget is set for: at most 4 (FP32 lines) or 2,
  // within the shared memory and the 2048 threads of an SM
  static constexpr int OCC0 = CB == 8 ? LAPS_PASSC_OCC_F32 : 2;
  static constexpr int OCC1 = (227 * 1024) / (SMEM + 1024) < OCC0 ? (227 * 1024) / (SMEM + 1024) : OCC0;
  static constexpr int OCC2 = 2048 / THREADS < OCC1 ? 2048 / THREADS : OCC1;
  static constexpr int OCC = OCC2 < 1 ? 1 : OCC2;
};

#ifndef LAPS_DD_SHARED_FFT
#define LAPS_DD_SHARED_FFT 1
#endif
#ifndef LAPS_PAIR_POINTS
#define LAPS_PAIR_POINTS 1
#endif
template <class T, class TS, int NX, int CFL, int INCOMP>
__global__ void __launch_bounds__(PassCCfg<NX, (int)sizeof(typename Store<T>::C)>::THREADS,
                                  PassCCfg<NX, (int)sizeof(typename Store<T>::C)>::OCC) k_passC(Bufs<T, TS> b, PassArgs a, PassK<T, TS> kk, const typename Store<T>::C* __restrict__ twx) {
  const PT<T>& pc = kk.pc;
  using C = typename Store<T>::C;
  using CF = PassCCfg<NX, (int)sizeof(C)>;
  using SR = typename Store<T>::R;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  if (a.st->halt) return;
  C* sc = reinterpret_cast<C*>(smem_raw);  // [row][field] lines of LC complex
  SR* sr = reinterpret_cast<SR*>(smem_raw);
  const Geo& g = a.g;
  const int nin = INCOMP ? 19 : (a.hall ? 11 : 8);
  // fluxes transformed, in order: the momentum flux tensor is symmetric (T_xy = T_yx,
  // T_xz = T_zx, T_yz = T_zy), so slots 6, 9, 10 are never needed; slots 0..2 are skipped
  // when the continuity term comes from the state
  const int* flist = INCOMP ? c_flist[2] : c_flist[a.mass_from_state ? 1 : 0];
  const int nfl = a.cfl == 2 ? 0 : (INCOMP ? 6 : (a.mass_from_state ? 13 : 16) - (a.aeb ? 0 : 1));
  long long row0 = (long long)blockIdx.x * CF::ROWS;  // row = z*ny + y
  const int lt = threadIdx.x % CF::TPL, lb = threadIdx.x / CF::TPL;
  // real values of point p (row p / NX, x = p % NX): field f at base + f * CF::FSTR
  auto point_base = [&](int p) -> SR* {
    const int rr = p / NX, x = p % NX;
    if constexpr (CF::PAIRED) return sr + 2 * ((rr >> 1) * CF::NF * CF::LCP + sm_idx<1>(x)) + (rr & 1);
    else return sr + 2 * rr * CF::NF * CF::LC + row_real_idx(x);
  };
  const int kk_in = g.kx_keep;
  // float-float 256-point rows: one (called) copy of the transform for both directions (pass
  // time -9 %: the kernel stalled on instruction fetch; FP64 rows, ALU-bound, lose 3 % and
  // keep both inlined copies)
  constexpr bool SHARED_FFT = LAPS_DD_SHARED_FFT && std::is_same<T, dd>::value && NX == 256 && CF::PAIRED;
  if constexpr (CF::PAIRED) {
    // ---- inverse x-transform of row pairs: Z = X_a + i X_b over the full line (the
    // imaginary parts of the DC and Nyquist terms are dropped, as the reference's c2r does)
    const int ltp = threadIdx.x % CF::TPLP, lbp = threadIdx.x / CF::TPLP;
    constexpr int NPAIR = CF::ROWS / 2;
    for (int L0 = 0; L0 < NPAIR * nin; L0 += CF::LBP) {
      const int L = L0 + lbp;
      const bool act = L < NPAIR * nin;
      const int pr = act ? L / nin : 0, f = act ? L % nin : 0;
      C* z = sc + (pr * CF::NF + f) * CF::LCP;
      if (act) {
        const C* xa = b.W2 + f * g.fsc + (row0 + 2 * pr) * g.kxp;
        pair_c2r<T, NX>(z, ltp, kk_in, xa, xa + g.kxp);
      }
      // a line and its threads stay within one warp until the physics (1024-point lines: two
      // warps, synchronised by block barriers every thread of the block reaches)
      if constexpr (CF::LWARP) __syncwarp();
      else __syncthreads();
      if constexpr (SHARED_FFT) fft_row_shared<T, NX, +1>(z, ltp, act, twx, 1);
      else fft_lines<T, NX, +1, 1, 0, CF::LWARP>(z, 0, ltp, act, twx, 1);
    }
  } else {
    // ---- c2r of the inputs, one half-length complex line per row
    for (int L0 = 0; L0 < CF::ROWS * nin; L0 += CF::LB) {
      int L = L0 + lb;
      bool act = L < CF::ROWS * nin;
      int rr = act ? L / nin : 0, f = act ? L % nin : 0;
      C* z = sc + (rr * CF::NF + f) * CF::LC;
      if (act) {
        const C* xin = b.W2 + f * g.fsc + (row0 + rr) * g.kxp;
        c2r_pre<T, CF::H>(z, lt, [&](int k) { return k < kk_in ? Store<T>::ldg(xin + k) : cx_zero<T>(); }, twx);
      }
      __syncwarp();  // a line and its threads stay within one warp until the physics
      fft_lines<T, CF::H, +1, 1, 0, true>(z, 0, lt, act, twx, 2);
    }
  }
  __syncthreads();
  constexpr int NQ = INCOMP ? 19 : 11;
  using PH = typename std::conditional<INCOMP, FluxI<T>, Flux<T>>::type;
  // ---- CFL minimum (vardt, mhd.f90:328-429), screened: every point in FP32 with the
  // approximate divide and square root, then only the points within 0.01 % of the block's
  // FP32 minimum (or FP32 NaN) in the state type TS.  The screened value of a point's bound is
  // within 1e-5 of its TS value, so the block's TS minimum is the one a full TS evaluation
  // gives.  Blocks also publish their FP32 minimum to the step's running minimum: a block
  // whose minimum lies above 1.0001 times a published one holds no point whose TS bound can be
  // the step's minimum and evaluates nothing in TS (the block with the smallest published
  // minimum always evaluates, and so does every block with an FP32 NaN).
  constexpr int MAXC = 32;
  __shared__ SR cand[CFL ? MAXC : 1][NQ];
  __shared__ int ncand, skip_ts;
  bool cand_late = false;  // block-uniform: the list waits for warp 0 at the end
  using PHS = typename std::conditional<INCOMP, FluxI<TS>, Flux<TS>>::type;
  const TS rfac = Real<TS>::from_d(a.st->rfac);  // radius / R0
  auto report = [&](TS tmin, bool nan_seen) {  // warp min, then one atomic per warp
    double dmin = Real<TS>::to_d(tmin);
    for (int o = 16; o > 0; o >>= 1) dmin = fmin(dmin, __shfl_xor_sync(0xffffffffu, dmin, o));
    const bool any_nan = __any_sync(0xffffffffu, nan_seen);
    if ((threadIdx.x & 31) == 0) {
      if (any_nan) atomicOr(&a.st->status, LAPS_STATUS_NAN);
      atomicMin(&a.st->cfl_bits, (unsigned long long)__double_as_longlong(dmin));
    }
  };
  // warp 0: the candidate list in TS
  auto eval_list = [&]() {
    if (threadIdx.x >= 32) return;
    TS tmin = Real<TS>::inf();
    bool nan_seen = false;
    if ((int)threadIdx.x < ncand) {
      TS qs[NQ];
#pragma unroll
      for (int f = 0; f < NQ; f++) qs[f] = f < nin ? Cvt<TS, T>::r(Store<T>::ld(&cand[threadIdx.x][f])) : kk.ps.zero;
      const TS d = PHS::cfl(qs, kk.ps, a.P, rfac);
      if (Real<TS>::isnan_(d)) nan_seen = true;
      else tmin = d;
    }
    report(tmin, nan_seen);
  };
  if (CFL) {
    using PHF = typename std::conditional<INCOMP, FluxI<float>, Flux<float>>::type;
    __shared__ float red32[32];
    const PT<float> pf = pt_float(pc);
    const float rfac_f = a.st->f_rfac;
    constexpr int PPT = (CF::ROWS * NX + CF::THREADS - 1) / CF::THREADS;  // points per thread
    float d32[PPT];
    float m32 = __int_as_float(0x7f800000);
    bool nan32 = false;
#pragma unroll
    for (int i = 0; i < PPT; i++) {
      const int p = threadIdx.x + i * CF::THREADS;
      d32[i] = m32;
      if (p < CF::ROWS * NX) {
        const SR* base = point_base(p);
        float qf[NQ];
#pragma unroll
        for (int f = 0; f < NQ; f++) qf[f] = f < nin ? Cvt<float, T>::r(Store<T>::ld(base + f * CF::FSTR)) : 0.f;
        d32[i] = PHF::cfl_screen(qf, pf, a.P, rfac_f);
        m32 = fminf(m32, d32[i]);
        nan32 |= isnan(d32[i]);
      }
    }
    // candidates: the points within 0.01 % of the block's FP32 minimum, and FP32 NaNs; their
    // inputs are copied to a list that one warp evaluates in TS after its other work
    if (threadIdx.x == 0) ncand = 0;
    for (int o = 16; o > 0; o >>= 1) m32 = fminf(m32, __shfl_xor_sync(0xffffffffu, m32, o));
    if ((threadIdx.x & 31) == 0) red32[threadIdx.x >> 5] = m32;
    const bool any_nan = __syncthreads_or(nan32) != 0;
    for (int w = 0; w < CF::THREADS / 32; w++) m32 = fminf(m32, red32[w]);
    const float thr = m32 * 1.0001f;
    if (threadIdx.x == 0) {
      // bounds are positive (or +inf), so their float bits order as unsigned integers
      bool skip = false;
      if (m32 >= 0.f) {
        const unsigned int old = atomicMin(&a.st->cfl32_bits, __float_as_uint(m32));
        skip = !any_nan && m32 > 1.0001f * __uint_as_float(old);
      }
      skip_ts = skip;
    }
#pragma unroll
    for (int i = 0; i < PPT; i++) {
      const int p = threadIdx.x + i * CF::THREADS;
      if (p >= CF::ROWS * NX || (!(d32[i] <= thr) && !isnan(d32[i]))) continue;
      const int slot = atomicAdd(&ncand, 1);
      if (slot < MAXC) {
        const SR* base = point_base(p);
#pragma unroll
        for (int f = 0; f < NQ; f++) cand[slot][f] = f < nin ? base[f * CF::FSTR] : SR{};
      }
    }
    __syncthreads();  // the list is complete; the physics may now overwrite the inputs
    const int nc = ncand;
    if (skip_ts) {
      // another block's FP32 minimum is below this block's by more than the screen's error
    } else if (nc <= MAXC) {
      // the list is evaluated by warp 0 at the end of the kernel, off the physics' barrier
      cand_late = true;
    } else {  // more candidates than the list holds: every thread evaluates its own
      TS tmin = Real<TS>::inf();
      bool nan_seen = false;
#pragma unroll
      for (int i = 0; i < PPT; i++) {
        const int p = threadIdx.x + i * CF::THREADS;
        if (p >= CF::ROWS * NX || (!(d32[i] <= thr) && !isnan(d32[i]))) continue;
        const SR* base = point_base(p);
        TS qs[NQ];
#pragma unroll
        for (int f = 0; f < NQ; f++) qs[f] = f < nin ? Cvt<TS, T>::r(Store<T>::ld(base + f * CF::FSTR)) : kk.ps.zero;
        const TS d = PHS::cfl(qs, kk.ps, a.P, rfac);
        if (Real<TS>::isnan_(d)) nan_seen = true;
        else tmin = Real<TS>::min_(tmin, d);
      }
      report(tmin, nan_seen);
      __syncthreads();  // before the physics overwrites the inputs
    }
  }
  if (nfl == 0) {
    if (CFL && cand_late) eval_list();
    return;
  }
  // ---- physics per point, in place (inputs and outputs of a point share its slots)
  T inv_tau, inv_rho0;
  if constexpr (std::is_same<T, float>::value) {
    inv_tau = a.st->f_inv_tau;
    inv_rho0 = a.st->f_inv_rho0;
  } else {
    inv_tau = Real<T>::from_d(a.st->inv_tau);
    inv_rho0 = Real<T>::from_d(a.st->inv_rho0);
  }
  if constexpr (LAPS_PAIR_POINTS && std::is_same<T, float>::value && CF::PAIRED) {
    // FP32 paired rows: the two rows of a pair share each complex slot (row 2p in .x, row
    // 2p+1 in .y), so one thread takes both points at an x, with one 8-byte load and one
    // 8-byte store per field (a warp then reads consecutive 8-byte slots: no bank conflict);
    // the first point's outputs wait in registers until the second point produces its own
    constexpr int NPAIR = CF::ROWS / 2;
    C* sc2 = reinterpret_cast<C*>(smem_raw);
#pragma unroll 1
    for (int p = threadIdx.x; p < NPAIR * NX; p += CF::THREADS) {
      const int pr = p / NX, xx = p - pr * NX;
      C* base = sc2 + pr * CF::NF * CF::LCP + sm_idx<1>(xx);
      T q0[NQ], q1[NQ];
#pragma unroll
      for (int f = 0; f < NQ; f++) {
        const cx<T> v = f < nin ? Store<T>::ldc(base + f * CF::LCP) : cx_zero<T>();
        q0[f] = v.re;
        q1[f] = v.im;
      }
      T o0[19];
      PH::eval(q0, [&](int k, T v) { o0[k] = v; }, pc, a.P, inv_tau, inv_rho0);
      PH::eval(q1, [&](int k, T v) { if ((c_fused >> k) & 1) Store<T>::stc(base + k * CF::LCP, cx<T>{o0[k], v}); }, pc, a.P, inv_tau, inv_rho0);
    }
  } else
#pragma unroll 1
  for (int p = threadIdx.x; p < CF::ROWS * NX; p += CF::THREADS) {
    SR* base = point_base(p);
    T q[NQ];
#pragma unroll
    for (int f = 0; f < NQ; f++) q[f] = f < nin ? Store<T>::ld(base + f * CF::FSTR) : pc.zero;
    PH::eval(q, [&](int k, T v) { if ((c_fused >> k) & 1) Store<T>::st(base + k * CF::FSTR, v); }, pc, a.P, inv_tau, inv_rho0);
  }
  __syncthreads();
  // ---- forward x-transforms of the fluxes
  const int sexp = -__ffs(NX) + 1;  // 1/nx
  if constexpr (CF::PAIRED) {
    const int ltp = threadIdx.x % CF::TPLP, lbp = threadIdx.x / CF::TPLP;
    constexpr int NPAIR = CF::ROWS / 2;
    for (int L0 = 0; L0 < NPAIR * nfl; L0 += CF::LBP) {
      const int L = L0 + lbp;
      const bool act = L < NPAIR * nfl;
      const int pr = act ? L / nfl : 0, f = act ? flist[L % nfl] : 0;
      C* z = sc + (pr * CF::NF + f) * CF::LCP;
      if constexpr (SHARED_FFT) fft_row_shared<T, NX, -1>(z, ltp, act, twx, 1);
      else fft_lines<T, NX, -1, 1, 0, CF::LWARP>(z, 0, ltp, act, twx, 1);
      if (act) {
        C* xa = b.W1 + f * g.fsc + (row0 + 2 * pr) * g.kxp;
        pair_r2c<T, NX>(z, ltp, kk_in, xa, xa + g.kxp, sexp);
      }
    }
  } else {
    for (int L0 = 0; L0 < CF::ROWS * nfl; L0 += CF::LB) {
      int L = L0 + lb;
      bool act = L < CF::ROWS * nfl;
      int rr = act ? L / nfl : 0, f = act ? flist[L % nfl] : 0;
      C* z = sc + (rr * CF::NF + f) * CF::LC;
      fft_lines<T, CF::H, -1, 1, 0, true>(z, 0, lt, act, twx, 2);
      if (act) {
        C* xo = b.W1 + f * g.fsc + (row0 + rr) * g.kxp;
        r2c_post<T, CF::H>(z, lt, [&](int k, cx<T> v) { if (k < kk_in) Store<T>::stc(xo + k, v); }, sexp, twx);
      }
    }
  }
  if (CFL && cand_late) eval_list();  // after this warp's share of the transforms
}

// Resident blocks per SM the register budget of passes D and E is set for (FP32 lines) and
// how they transform their two input tiles: one after the other with 6 blocks (the shared-
// memory limit of two 16 KB tiles) measured best at 256^3 (passes D + E -0.06 ms per step).
// Transforming both tiles together (LAPS_COL_PAIR_FFT=1: fft_lines_pair, half the barriers
// but twice the live elements per thread) needs 96 registers and runs 5 blocks; the pairs
// with 6 or 7 blocks spilled (+9 %, +11 %).  Both macros override the choice at build time.
#ifndef LAPS_MINB_COL
#define LAPS_MINB_COL 6
#endif
#ifndef LAPS_COL_PAIR_FFT
#define LAPS_COL_PAIR_FFT 0
#endif
// (float-float: 4 and FP64: 3, the budgets the compiler picks for them without a bound)
template <class T> struct ColOcc {
  static constexpr int V = sizeof(typename Store<T>::C) == 8 ? LAPS_MINB_COL : (std::is_same<T, double>::value ? 3 : 4);
};
// the same registers per thread for longer columns, whose blocks have more threads (512- and
// 1024-point columns: 256 and 512 threads; a fixed block count would leave 32-64 registers
// and spill)
template <class T, int N> struct ColOccN {
  static constexpr int W = ColOcc<T>::V * 128 / Col<T, N>::THREADS;
  static constexpr int V = W < 1 ? 1 : W;
};

// ============================================================================ pass D
// forward y-FFT of the fluxes with the kx, ky parts of the spectral right-hand side folded
// in (calc_rhs, mhdrhs.f90:206-233), leaving only the kz parts for pass E.  Compressible
// output slots:
//   0 Q1 = -(i ax F1 + i ay F2)      1 F3
//   2 Q2 = -(i ax F4 + i ay F5)      3 F6
//   4 Q3 = -(i ax F7 + i ay F8)      5 F9
//   6 Q4 = -(i ax F10 + i ay F11)    7 F12
//   8 Ex   9 Ey   10 P7 = i ay Ex - i ax Ey   11 P5 = -i ay Ez   12 P6 = i ax Ez
//   13 Q8 = -(i ax F16 + i ay F17) + Expand   14 F18
// Incompressible output slots: 0..2 the pressure flux, 3 Ex, 4 Ey, 5 P7, 6 P5, 7 P6.
// One group per blockIdx.z; tile: kx0..kx0+7, one z plane; reads all y of W1, writes kept
// ky rows of W2.
struct DGroup { signed char in[3], kind, out; };
// kinds: Q:    out = -(i ax F_a + i ay F_b)
//        COPY: out = F_a
//        EXY:  out, out+1, out+2 = Ex, Ey, i ay Ex - i ax Ey
//        EZ:   out, out+1 = -i ay Ez, i ax Ez
//        Q8:   out = -(i ax F_a + i ay F_b) (+ expansion term F_c)
//        QQ:   (F3, F4 = F6, F7) -> out = Q2 = -(i ax Txx + i ay Tyx), out+2 = Q3 = -(i ax Txy + i ay Tyy)
//        T3:   (F5 = F9, F8 = F10, F11) -> out = Tzx, out+2 = Tzy, out+3 = Q4 = -(i ax Txz + i ay Tyz), out+4 = Tzz
enum { DG_Q = 0, DG_COPY, DG_EXY, DG_EZ, DG_Q8, DG_QQ, DG_T3 };
__constant__ DGroup c_dgroups[2][8] = {
    {{{0, 1, -1}, DG_Q, 0}, {{2, -1, -1}, DG_COPY, 1}, {{3, 4, 7}, DG_QQ, 2}, {{5, 8, 11}, DG_T3, 3},
     {{12, 13, -1}, DG_EXY, 8}, {{14, -1, -1}, DG_EZ, 11}, {{15, 16, 18}, DG_Q8, 13}, {{17, -1, -1}, DG_COPY, 14}},
    {{{0, -1, -1}, DG_COPY, 0}, {{1, -1, -1}, DG_COPY, 1}, {{2, -1, -1}, DG_COPY, 2}, {{3, 4, -1}, DG_EXY, 3},
     {{5, -1, -1}, DG_EZ, 6}}};

template <class T, class TS, int NY>
__global__ void __launch_bounds__(Col<T, NY>::THREADS, ColOccN<T, NY>::V)
    k_passD(Bufs<T, TS> b, PassArgs a, PassK<T, TS> kk, const typename Store<T>::C* __restrict__ twy,
            const __grid_constant__ CUtensorMap tmap) {
  const PT<T>& pc = kk.pc;
  const KTab<T>& K = kk.K;
  using CL = Col<T, NY>;
  using C = typename Store<T>::C;
  extern __shared__ __align__(128) unsigned char smem_tma[];  // 128-byte aligned: TMA destinations
  __shared__ __align__(8) uint64_t tbar[2];
  if (a.st->halt) return;
  ColCtx<T, NY, 2> x(reinterpret_cast<C*>(smem_tma));
  const Geo& g = a.g;
  const DGroup grp = c_dgroups[a.P.variant == LAPS_VARIANT_3DI ? 1 : 0][blockIdx.z + (a.mass_from_state ? 2 : 0)];
  int kx = blockIdx.x * TX + x.c;
  int z = blockIdx.y * CL::NTILE + x.tl;
  bool ok = kx < g.kx_keep && z < g.nz;
  long long col = (long long)z * g.ny * g.kxp + kx;
  T rr = Real<T>::from_d(a.st->r_ratio);
  const int sexp = -__ffs(NY) + 1;
  const int kind = grp.kind;
  const int nin = grp.in[1] < 0 ? 1 : (grp.in[2] < 0 || (kind == DG_Q8 && !a.aeb) ? 2 : 3);
  C* ob = b.W2 + col + grp.out * g.fsc;
  // Input tiles come by TMA (one copy per tile and 256-line box, issued by thread 0): inputs
  // 0 and 1 at the start into buffers 0 and 1, a third into the buffer its group has finished
  // with.  FP32 lines transform inputs 0 and 1 together; wider types one after the other.
  TileLoad tl;
  tl.init(tbar);
  auto issue = [&](int k, int bi) {
    if (threadIdx.x == 0) {
      constexpr int EW = (int)(sizeof(C) / 8), YB = NY < 256 ? NY : 256;
      const int z0 = blockIdx.y * CL::NTILE;
      const int nt = g.nz - z0 < CL::NTILE ? g.nz - z0 : CL::NTILE;
      tl.expect(bi, (uint32_t)(nt * NY * TX * (int)sizeof(C)));
      for (int t = 0; t < nt; t++) {
        C* dst = reinterpret_cast<C*>(smem_tma) + (t * 2 + bi) * NY * TX;  // tile t, buffer bi
        for (int y0 = 0; y0 < NY; y0 += YB) tl.copy(bi, dst + y0 * TX, &tmap, blockIdx.x * TX * EW, y0, grp.in[k] * g.nz + z0 + t);
      }
    }
  };
  constexpr bool PAIR = sizeof(C) == 8 && LAPS_COL_PAIR_FFT;
  // one shared-memory tile (1024-point columns of 16-byte elements): the inputs come one
  // after the other into buffer 0, and the tile a later input would have found in the other
  // buffer is kept as each thread's own elements in registers (rb)
  constexpr bool ONEBUF = col_one_buffer<T, NY>();
  static_assert(!ONEBUF || CL::NTILE == 1, "one buffer: single-tile blocks (ColCtx lays tiles out with two buffers)");
  cx<T> rb[2][ONEBUF ? CL::EPT : 1];
  auto vget = [&](int vb, int cur, int m) -> cx<T> {
    if constexpr (ONEBUF) return vb == cur ? Store<T>::ldc(x.at(0, m)) : rb[vb][m];
    else return Store<T>::ldc(x.at(vb, m));
  };
  auto vput0 = [&](int cur, int m, cx<T> v) {
    if constexpr (ONEBUF) {
      if (cur == 0) Store<T>::stc(x.at(0, m), v);
      else rb[0][m] = v;
    } else {
      Store<T>::stc(x.at(0, m), v);
    }
  };
  issue(0, 0);
  if (nin > 1 && !ONEBUF) issue(1, 1);
  if (PAIR) {
    if (!tl.wait(0, a.st) || (nin > 1 && !tl.wait(1, a.st))) return;
    fft_lines_pair<T, NY, -1, TX, 1>(x.buf(0), x.buf(1), nin > 1, x.c, x.t, twy, 1);
  }
#pragma unroll 1
  for (int k = 0; k < nin; k++) {
    int cur = 0;  // the (virtual) buffer input k is in
    if (k == 2 || !PAIR) {
      const int bi = k == 1 || (k == 2 && kind == DG_Q8) ? 1 : 0;
      cur = bi;
      if constexpr (ONEBUF) {
        if (k > 0) {  // buffer 0's earlier contents were read by the threads
          if (threadIdx.x == 0) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          issue(k, 0);
        }
        if (!tl.wait(0, a.st)) return;
        fft_lines<T, NY, -1, TX, 1>(x.buf(0), x.c, x.t, true, twy, 1);
      } else {
        if (k == 2) {  // the buffer's earlier contents were read and written by the threads
          if (threadIdx.x == 0) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          issue(2, bi);
        }
        if (!tl.wait(bi, a.st)) return;
        fft_lines<T, NY, -1, TX, 1>(x.buf(bi), x.c, x.t, true, twy, 1);
      }
    }
    if (ok) {
#pragma unroll 2
      for (int m = 0; m < CL::EPT; m++) {
        const int ky = x.j(m);
        T ax, ay, az;
        kfac(K, a.P, pc, rr, kx, ky, 0, ax, ay, az);
        const bool st_ok = g.ky_in(ky);
        C* o = ob + (long long)ky * g.kxp;
        cx<T> v0 = vget(0, cur, m), v1 = cx_zero<T>();
        if (k > 0) v1 = vget(1, cur, m);
        if (kind == DG_Q8) {
          if (k == 1) {  // fold the two fluxes into buffer 0, unscaled
            vput0(cur, m, -(mul_i(v0, ax) + mul_i(v1, ay)));
            if (nin == 2 && st_ok) {
              cx<T> q = -(mul_i(v0, ax) + mul_i(v1, ay));
              Store<T>::stc(o, {Real<T>::mul_pow2(q.re, sexp), Real<T>::mul_pow2(q.im, sexp)});
            }
          } else if (k == 2 && st_ok) {
            cx<T> q = v0 + v1;
            Store<T>::stc(o, {Real<T>::mul_pow2(q.re, sexp), Real<T>::mul_pow2(q.im, sexp)});
          }
          continue;
        }
        v0 = {Real<T>::mul_pow2(v0.re, sexp), Real<T>::mul_pow2(v0.im, sexp)};
        v1 = {Real<T>::mul_pow2(v1.re, sexp), Real<T>::mul_pow2(v1.im, sexp)};
        if (!st_ok) continue;
        switch (kind) {
          case DG_Q: if (k == 1) Store<T>::stc(o, -(mul_i(v0, ax) + mul_i(v1, ay))); break;
          case DG_COPY: Store<T>::stc(o, v0); break;
          case DG_EXY:
            if (k == 1) {
              Store<T>::stc(o, v0);
              Store<T>::stc(o + g.fsc, v1);
              Store<T>::stc(o + 2 * g.fsc, mul_i(v0, ay) - mul_i(v1, ax));
            }
            break;
          case DG_EZ:
            Store<T>::stc(o, -mul_i(v0, ay));
            Store<T>::stc(o + g.fsc, mul_i(v0, ax));
            break;
          case DG_QQ:  // buffer 0: Txx then Tyy; buffer 1: Tyx (= Txy)
            if (k == 1) Store<T>::stc(o, -(mul_i(v0, ax) + mul_i(v1, ay)));
            else if (k == 2) Store<T>::stc(o + 2 * g.fsc, -(mul_i(v1, ax) + mul_i(v0, ay)));
            break;
          default:  // DG_T3: buffer 0: Tzx (= Txz) then Tzz; buffer 1: Tzy (= Tyz)
            if (k == 0) Store<T>::stc(o, v0);
            else if (k == 1) {
              Store<T>::stc(o + 2 * g.fsc, v1);
              Store<T>::stc(o + 3 * g.fsc, -(mul_i(v0, ax) + mul_i(v1, ay)));
            } else Store<T>::stc(o + 4 * g.fsc, v0);
            break;
        }
      }
      if constexpr (ONEBUF) {  // keep this input's transform before the next one overwrites it
#pragma unroll
        for (int m = 0; m < CL::EPT; m++) rb[cur][m] = Store<T>::ldc(x.at(0, m));
      }
    }
    __syncthreads();
  }
}

// ============================================================================ pass E
#ifndef LAPS_E_CHUNK
#define LAPS_E_CHUNK 4  // elements whose state and RK-register loads pass E issues together
#endif
// Per-element tail of the spectral right-hand side and the time advance of variable v:
// expansion damping (mhdrhs.f90:235-251), explicit diffusion (:253-275), the RK3 update with
// implicit diffusion (rktmod.f90:34-62) and the dealias mask or filter (dealiasing.f90:70-113).
// T: the state type (the update's arithmetic); TR: the type of the RK register, which holds
// the previous stages' right-hand side (the transforms' type: FP32 in the FP32-transform
// modes, where the right-hand side carries FP32 accuracy anyway)
// u / d of the implicit diffusion step: a float-float state takes one reciprocal and two
// products instead of two float-float divisions (roundings of ~2^-48, far inside the mode's
// 1e-12 bound; LAPS_DD_RECIP=0 restores the divisions); FP64 divides as the reference
template <class T> __device__ __forceinline__ cx<T> implicit_div(cx<T> u, T d) {
  if constexpr (LAPS_DD_RECIP && std::is_same<T, dd>::value) {
    const T r = Real<T>::recip(d);
    return {u.re * r, u.im * r};
  } else {
    return {u.re / d, u.im / d};
  }
}

template <class T, class TR = T>
struct RkCtx {
  using CR = typename Store<TR>::C;
  const Geo* g;
  const Phys* P;
  const PT<T>* pc;
  const KTab<T>* K;
  T cc, ddc, ts, inv_tau, rr;
  int stage, store_rk, plain, rhs_only;
  __device__ __forceinline__ T k2(int kx, int ky, int kz) const {
    if (P->corot && !plain) return ksq(*K, *P, *pc, rr, kx, ky, kz);
    return (K->kx2[kx] + K->ky2[ky]) + K->kz2[kz];
  }
  // the RK register of an element as the update needs it: read after stage 0 only (coherent
  // load: the update rewrites it)
  __device__ __forceinline__ cx<T> r_of(const CR* R) const {
    return stage > 0 ? cvtc<T>(Store<TR>::ldc(R)) : cx_zero<T>();
  }
  __device__ __forceinline__ void update(int v, cx<T> fnl, cx<T> u, typename Store<T>::C* U, CR* R, T k2, int kx, int ky,
                                         int kz) const {
    update(v, fnl, u, r_of(R), U, R, k2, kx, ky, kz);
  }
  // u: the element's state, r: its RK register (from r_of), both read before the call
  __device__ __forceinline__ void update(int v, cx<T> fnl, cx<T> u, cx<T> r, typename Store<T>::C* U, CR* R, T k2, int kx,
                                         int ky, int kz) const {
    const bool mom = v >= 1 && v <= 3, mag = v >= 4 && v <= 6;
    if (P->aeb && (P->ebm_mask >> v & 1)) fnl = fnl - u * (pc->ebm[v] * inv_tau);
    if (mom && P->visc && P->visc_exp) fnl = fnl - u * (pc->nu * k2);
    if (mag && P->resis && P->resis_exp && !(P->cons_bg && kx == 0 && kz == 0)) fnl = fnl - u * (pc->eta * k2);
    if (rhs_only) {  // calc_rhs alone: fnl with the expansion and explicit-diffusion terms
      Store<TR>::stc(R, cvtc<TR>(fnl));
      return;
    }
    cx<T> un = fnl * cc + u;
    if (stage > 0) un = (fnl * cc + r * ddc) + u;
    if (store_rk) Store<TR>::stc(R, cvtc<TR>(fnl));
    if (mom && P->visc && !P->visc_exp) {
      T d = ts * k2 * pc->nu + pc->one;
      un = implicit_div(un, d);
    }
    if (mag && P->resis && !P->resis_exp) {
      T d = ts * k2 * pc->eta + pc->one;
      un = implicit_div(un, d);
    }
    if (P->dealias == 1 || P->dealias == 3) {
      if (kx >= K->kxlim[kz * g->ny + ky]) un = cx_zero<T>();
    } else if (P->dealias == 2) {
      un = ((un * K->fx[kx]) * K->fy[ky]) * K->fz[kz];
    }
    Store<T>::stc(U, un);
  }
  // The same update when the right-hand side is an FP32 value (FP32-transform modes).  The
  // implicit step (u + inc) / (1 + x), x = dt_sub k^2 nu (or eta), is rewritten exactly as
  // u + (inc - x u) / (1 + x): everything but the accumulation into u is a correction of the
  // size of the FP32 right-hand side and is formed in FP32 (expansion / explicit-diffusion
  // terms, the increment cc fnl + ddc r, the diffusion decrement and its factor); the
  // accumulation u + correction, which carries the state itself, stays in the state type.
  // This keeps the state type's arithmetic to one addition per component (no division in
  // the state type, whose FP64 form issues ~70x slower than FP32 on this GPU).
  // cf: the FP32 constants (ebm, nu, eta); k2f, tsf: k^2 and the sub-step in FP32.
  __device__ __forceinline__ void update_f32(int v, cx<float> fnl, cx<T> u, cx<float> r, typename Store<T>::C* U, CR* R, float k2f,
                                             int kx, int ky, int kz, const PT<float>& cf, float ccf, float ddcf,
                                             float itf, float tsf) const {
    const bool mom = v >= 1 && v <= 3, mag = v >= 4 && v <= 6;
    const cx<float> uf = IncCvt<T>::to_f32(u);
    if (P->aeb && (P->ebm_mask >> v & 1)) fnl = fnl - uf * (cf.ebm[v] * itf);
    if (mom && P->visc && P->visc_exp) fnl = fnl - uf * (cf.nu * k2f);
    if (mag && P->resis && P->resis_exp && !(P->cons_bg && kx == 0 && kz == 0)) fnl = fnl - uf * (cf.eta * k2f);
    if (rhs_only) {
      Store<TR>::stc(R, cvtc<TR>(fnl));
      return;
    }
    cx<float> inc = fnl * ccf;
    if (stage > 0) inc = fnl * ccf + r * ddcf;
    if (store_rk) Store<TR>::stc(R, cvtc<TR>(fnl));
    const bool vimp = mom && P->visc && !P->visc_exp, rimp = mag && P->resis && !P->resis_exp;
    if (vimp || rimp) {
      const float x = tsf * k2f * (vimp ? cf.nu : cf.eta);
      const float id = 1.0f / (1.0f + x);
      inc = (inc - uf * x) * id;
    }
    cx<T> un;
    if ((P->dealias == 1 || P->dealias == 3) && kx >= K->kxlim[kz * g->ny + ky]) {
      un = cx_zero<T>();
    } else {
      un = u + IncCvt<T>::from_f32(inc);
      if (P->dealias == 2) un = ((un * K->fx[kx]) * K->fy[ky]) * K->fz[kz];
    }
    Store<T>::stc(U, un);
  }
};

template <class TR, class T>
__device__ __forceinline__ RkCtx<T, TR> rk_ctx(const PassArgs& a, const PT<T>& pc, const KTab<T>& K) {
  RkCtx<T, TR> r;
  r.g = &a.g; r.P = &a.P; r.pc = &pc; r.K = &K;
  r.stage = a.stage;
  r.store_rk = a.store_rk;
  if constexpr (std::is_same<T, float>::value) {  // the step state's FP32 copies
    r.cc = a.st->f_cc[a.stage];
    r.ddc = a.st->f_ddc[a.stage];
    r.ts = a.st->f_ts[a.stage];
    r.inv_tau = a.st->f_inv_tau;
    r.rr = a.st->f_r_ratio;
  } else {
    r.cc = Real<T>::from_d(a.st->cc[a.stage]);
    r.ddc = Real<T>::from_d(a.st->ddc[a.stage]);
    r.ts = Real<T>::from_d(a.st->ts[a.stage]);
    r.inv_tau = Real<T>::from_d(a.st->inv_tau);
    r.rr = Real<T>::from_d(a.st->r_ratio);
  }
  r.plain = a.st->ksq_plain;
  r.rhs_only = a.rhs_only;
  return r;
}

// Compressible: forward z-FFT with the kz parts of the right-hand side, then the tail and
// the time advance of variable v = blockIdx.z.  Tile: kx0..kx0+7, one kept ky row; reads all
// z of W2, writes kept kz of U (and R).
template <class T, class TS, int NZ>
__global__ void __launch_bounds__(Col<T, NZ>::THREADS, ColOccN<T, NZ>::V)
    k_passE(Bufs<T, TS> b, PassArgs a, PassK<T, TS> kk, const typename Store<T>::C* __restrict__ twz,
            const __grid_constant__ CUtensorMap tmap, const __grid_constant__ CUtensorMap tmu,
            const __grid_constant__ CUtensorMap tmr) {
  const PT<T>& pc = kk.pc;
  const KTab<T>& K = kk.K;
  using CL = Col<T, NZ>;
  using C = typename Store<T>::C;
  extern __shared__ __align__(128) unsigned char smem_tma[];  // 128-byte aligned: TMA destinations
  __shared__ __align__(8) uint64_t tbar[2];
  if (a.st->halt) return;
  ColCtx<T, NZ, 2> x(reinterpret_cast<C*>(smem_tma));
  const Geo& g = a.g;
  const int v = blockIdx.z + a.e_first;
  int kx = blockIdx.x * TX + x.c;
  int r = blockIdx.y * CL::NTILE + x.tl;
  bool ok = kx < g.kx_keep && r < g.nky();
  int ky = ok ? g.ky_of(r) : 0;
  long long col = (long long)ky * g.kxp + kx;
  long long zs = (long long)g.ny * g.kxp;
  const int sexp = -__ffs(NZ) + 1;
  // inputs per variable: first (plain), second (times s * i kz), s = +-1 or 0 (none; also
  // in 2-D, where kz = 0)
  const int in1 = v == 4 ? 11 : v == 5 ? 12 : v == 6 ? 10 : v == 7 ? 13 : 2 * v;
  const int in2 = (v == 6 || a.P.two_d) ? -1 : v == 4 ? 9 : v == 5 ? 8 : v == 7 ? 14 : 2 * v + 1;
  const int nin = in2 < 0 ? 1 : 2;  // (the continuity update from the momentum is k_mass_rk)
  // Both input tiles come by TMA, issued at the start by thread 0 (tiles of 128-byte
  // multiples; a 2-D run's one-point z lines load through the threads instead)
  constexpr bool TMA = (NZ * TX * (int)sizeof(C)) % 128 == 0;
  if constexpr (TMA) {
    TileLoad tl;
    tl.init(tbar);
    if (threadIdx.x == 0) {
      constexpr int EW = (int)(sizeof(C) / 8), ZB = NZ < 256 ? NZ : 256;
      const int r0 = blockIdx.y * CL::NTILE;
      const int nt = g.nky() - r0 < CL::NTILE ? g.nky() - r0 : CL::NTILE;
      for (int k = 0; k < nin; k++) {
        tl.expect(k, (uint32_t)(nt * NZ * TX * (int)sizeof(C)));
        const int fin = k == 0 ? in1 : in2;
        for (int t = 0; t < nt; t++) {
          C* dst = reinterpret_cast<C*>(smem_tma) + (t * 2 + k) * NZ * TX;  // tile t, buffer k
          const int kyt = g.ky_of(r0 + t);
          for (int z0 = 0; z0 < NZ; z0 += ZB) tl.copy(k, dst + z0 * TX, &tmap, blockIdx.x * TX * EW, kyt, fin * g.nz + z0);
        }
      }
      // FP32 lines: the kept rows of the state and of the RK register this block updates
      // after its transform go into L2 now, so that their loads after the transform hit L2
      // (tmu / tmr boxes are the kept-row boxes of a.g; the RK register is not read in the
      // first stage).  Measured at 256^3: FP32 lines -3 % pass time; float-float +8 %, so not
      // there.
      using CSP = typename Store<TS>::C;
      constexpr int EWU = (int)(sizeof(CSP) / 8);
      const KeptCopies kp(g.kz_lo, g.kz_hi, NZ, 1);
      const int npf = sizeof(C) == 8 && !(a.sched & LAPS_SCHED_NO_PREFETCH_E) ? kp.count(NZ) : 0;
      for (int t = 0; t < nt; t++) {
        const int kyt = g.ky_of(r0 + t);
        for (int i = 0; i < npf; i++) {
          const int z0 = kp.start(i, NZ);
          tma_prefetch_3d(&tmu, blockIdx.x * TX * EWU, kyt, v * g.nz + z0);
          if (a.stage > 0 && !a.rhs_only) tma_prefetch_3d(&tmr, blockIdx.x * TX * EW, kyt, v * g.nz + z0);
        }
      }
    }
    if (!tl.wait(0, a.st) || (nin > 1 && !tl.wait(1, a.st))) return;
  } else {
#pragma unroll 1
    for (int k = 0; k < nin; k++) {
      const C* in = b.W2 + (k == 0 ? in1 : in2) * g.fsc + col;
#pragma unroll
      for (int m = 0; m < CL::EPT; m++) {
        cx<T> w = ok ? Store<T>::ldg(in + x.j(m) * zs) : cx_zero<T>();
        Store<T>::stc(x.at(k, m), w);
      }
    }
    __syncthreads();
  }
  if constexpr (sizeof(C) == 8 && LAPS_COL_PAIR_FFT) {  // FP32 lines: the two inputs transformed together
    fft_lines_pair<T, NZ, -1, TX, 1>(x.buf(0), x.buf(1), nin > 1, x.c, x.t, twz, 1);
  } else {
    fft_lines<T, NZ, -1, TX, 1>(x.buf(0), x.c, x.t, true, twz, 1);
    if (nin > 1) fft_lines<T, NZ, -1, TX, 1>(x.buf(1), x.c, x.t, true, twz, 1);
  }
  if (!ok) return;
  using CS = typename Store<TS>::C;
  const RkCtx<TS, T> rk = rk_ctx<T>(a, kk.ps, kk.KS);
  // FP32 transforms with a wider state: FP32 increments (RkCtx::update_f32), k^2 from the
  // FP32 tables
  constexpr bool F32INC = std::is_same<T, float>::value && !std::is_same<TS, float>::value;
  const RkCtx<T, T> rkf = rk_ctx<T>(a, kk.pc, kk.K);
  const float ccf = a.st->f_cc[a.stage], ddcf = a.st->f_ddc[a.stage], itf = a.st->f_inv_tau;
  const float tsf = a.st->f_ts[a.stage];
  const bool need_k2 = (v >= 1 && v <= 3 && a.P.visc) || (v >= 4 && v <= 6 && a.P.resis);
  CS* U = b.U + v * g.fsc + col;
  C* R = b.R + v * g.fsc + col;
  // elements in chunks of CH: the state and RK-register loads of a chunk are issued together
  // ahead of its arithmetic (the update's stores may alias them as far as the compiler knows)
  constexpr int CH = CL::EPT < LAPS_E_CHUNK ? CL::EPT : LAPS_E_CHUNK;
  // the RK register as the update reads it: FP32 as stored for FP32 increments, else in TS
  using RV = typename std::conditional<F32INC, float, TS>::type;
#pragma unroll 1
  for (int m0 = 0; m0 < CL::EPT; m0 += CH) {
    cx<TS> uo[CH];
    cx<RV> ro[CH];
#pragma unroll
    for (int i = 0; i < CH; i++) {
      const int kz = x.j(m0 + i);
      const long long idx = kz * zs;
      const bool in = g.kz_in(kz);
      uo[i] = in ? Store<TS>::ldc(U + idx) : cx_zero<TS>();
      if constexpr (F32INC) ro[i] = in && a.stage > 0 ? Store<T>::ldc(R + idx) : cx_zero<float>();
      else ro[i] = in ? rk.r_of(R + idx) : cx_zero<TS>();
    }
#pragma unroll
    for (int i = 0; i < CH; i++) {
      const int m = m0 + i;
      const int kz = x.j(m);
      if (!g.kz_in(kz)) continue;
      const long long idx = kz * zs;
      cx<T> f = Store<T>::ldc(x.at(0, m));
      f = {Real<T>::mul_pow2(f.re, sexp), Real<T>::mul_pow2(f.im, sexp)};
      if (nin > 1) {
        cx<T> w = Store<T>::ldc(x.at(1, m));
        w = mul_i(cx<T>{Real<T>::mul_pow2(w.re, sexp), Real<T>::mul_pow2(w.im, sexp)}, K.kzd[kz]);
        f = v == 4 ? f + w : f - w;
      }
      if constexpr (F32INC) {
        const float k2f = need_k2 ? Cvt<float, T>::r(rkf.k2(kx, ky, kz)) : 0.0f;
        rk.update_f32(v, f, uo[i], ro[i], U + idx, R + idx, k2f, kx, ky, kz, pc, ccf, ddcf, itf, tsf);
      } else {
        TS k2 = need_k2 ? rk.k2(kx, ky, kz) : kk.ps.zero;
        rk.update(v, cvtc<TS>(f), uo[i], ro[i], U + idx, R + idx, k2, kx, ky, kz);
      }
    }
  }
}

// Pass E of a 2-D run (nz = 1: the z transform is the identity): the same per-element tail
// and time advance as k_passE, over the kept (kx, ky) elements of variable
// v = blockIdx.y + e_first, read straight from W2 (k_passE's column tiles would hold one
// element per thread here); a flat 32-bit index over the kept elements, split by FastDiv.
template <class T, class TS>
__global__ void __launch_bounds__(256) k_passE2d(Bufs<T, TS> b, PassArgs a, PassK<T, TS> kk, FastDiv dkx) {
  if (a.st->halt) return;
  using CS = typename Store<TS>::C;
  using C = typename Store<T>::C;
  const Geo& g = a.g;
  const int v = blockIdx.y + a.e_first;
  const int in1 = v == 4 ? 11 : v == 5 ? 12 : v == 6 ? 10 : v == 7 ? 13 : 2 * v;
  const RkCtx<TS, T> rk = rk_ctx<T>(a, kk.ps, kk.KS);
  constexpr bool F32INC = std::is_same<T, float>::value && !std::is_same<TS, float>::value;
  const RkCtx<T, T> rkf = rk_ctx<T>(a, kk.pc, kk.K);
  const float ccf = a.st->f_cc[a.stage], ddcf = a.st->f_ddc[a.stage], itf = a.st->f_inv_tau;
  const float tsf = a.st->f_ts[a.stage];
  const bool need_k2 = (v >= 1 && v <= 3 && a.P.visc) || (v >= 4 && v <= 6 && a.P.resis);
  const C* W = b.W2 + in1 * g.fsc;
  CS* U = b.U + v * g.fsc;
  C* R = b.R + v * g.fsc;
  const unsigned tot = dkx.d * (unsigned)g.nky();  // < 2^31 for nz = 1
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < tot; i += gridDim.x * blockDim.x) {
    const unsigned r = dkx.div(i);
    const int kx = (int)(i - r * dkx.d);
    const int ky = g.ky_of((int)r);
    const long long idx = (long long)ky * g.kxp + kx;
    const cx<T> f = Store<T>::ldg(W + idx);
    const cx<TS> u = Store<TS>::ldc(U + idx);
    if constexpr (F32INC) {
      const cx<float> r = a.stage > 0 ? Store<T>::ldc(R + idx) : cx_zero<float>();
      const float k2f = need_k2 ? Cvt<float, T>::r(rkf.k2(kx, ky, 0)) : 0.0f;
      rk.update_f32(v, f, u, r, U + idx, R + idx, k2f, kx, ky, 0, kk.pc, ccf, ddcf, itf, tsf);
    } else {
      const cx<TS> r = rk.r_of(R + idx);
      TS k2 = need_k2 ? rk.k2(kx, ky, 0) : kk.ps.zero;
      rk.update(v, cvtc<TS>(f), u, r, U + idx, R + idx, k2, kx, ky, 0);
    }
  }
}

// Continuity update when the mass flux is the momentum (PassArgs::mass_from_state):
// fnl(rho) = -i k . (rho u)^ read from the state (mhdrhs.f90:206-209), then the tail and the
// time advance of rho for every kept element.  Launched before pass E updates the momentum.
template <class T, class TS, class IDX>
__global__ void __launch_bounds__(256) k_mass_rk(Bufs<T, TS> b, PassArgs a, PassK<T, TS> kk, FastDiv dkx, FastDiv dky) {
  if (a.st->halt) return;
  using CS = typename Store<TS>::C;
  const Geo& g = a.g;
  const RkCtx<TS, T> rk = rk_ctx<T>(a, kk.ps, kk.KS);
  constexpr bool F32INC = std::is_same<T, float>::value && !std::is_same<TS, float>::value;
  const float ccf = a.st->f_cc[a.stage], ddcf = a.st->f_ddc[a.stage], itf = a.st->f_inv_tau;
  const float tsf = a.st->f_ts[a.stage], rrf = a.st->f_r_ratio;
  // flat index over the kept elements: 32-bit, split by FastDiv, whenever the count allows
  // (IDX unsigned), else 64-bit division
  const IDX nkx = (IDX)g.kx_keep, nky = (IDX)g.nky();
  const IDX tot = nkx * nky * (IDX)g.nkz();
  for (IDX i = blockIdx.x * (IDX)blockDim.x + threadIdx.x; i < tot; i += (IDX)gridDim.x * blockDim.x) {
    int kx, ky, kz;
    if constexpr (std::is_same<IDX, unsigned>::value) {
      const unsigned r = dkx.div(i), q = dky.div(r);
      kx = (int)(i - r * dkx.d);
      ky = g.ky_of((int)(r - q * dky.d));
      kz = g.kz_of((int)q);
    } else {
      kx = (int)(i % nkx);
      const IDX r = i / nkx;
      ky = g.ky_of((int)(r % nky));
      kz = g.kz_of((int)(r / nky));
    }
    const long long idx = ((long long)kz * g.ny + ky) * g.kxp + kx;
    const cx<TS> m1 = Store<TS>::ldc(b.U + 1 * g.fsc + idx), m2 = Store<TS>::ldc(b.U + 2 * g.fsc + idx),
                 m3 = Store<TS>::ldc(b.U + 3 * g.fsc + idx);
    const cx<TS> u0 = Store<TS>::ldc(b.U + idx);
    if constexpr (F32INC) {
      // the right-hand side in FP32 (the mass flux's transform is FP32 in this mode), the
      // accumulation in the state type (RkCtx::update_f32)
      const cx<float> r0 = a.stage > 0 ? Store<T>::ldc(b.R + idx) : cx_zero<float>();
      float ax, ay, az;
      kfac(kk.K, a.P, kk.pc, rrf, kx, ky, kz, ax, ay, az);
      const cx<float> fm1 = IncCvt<TS>::to_f32(m1), fm2 = IncCvt<TS>::to_f32(m2), fm3 = IncCvt<TS>::to_f32(m3);
      const cx<float> fnl = -((mul_i(fm1, ax) + mul_i(fm2, ay)) + mul_i(fm3, az));
      rk.update_f32(0, fnl, u0, r0, b.U + idx, b.R + idx, 0.0f, kx, ky, kz, kk.pc, ccf, ddcf, itf, tsf);
    } else {
      const cx<TS> r0 = rk.r_of(b.R + idx);
      TS ax, ay, az;
      kfac(kk.KS, a.P, kk.ps, rk.rr, kx, ky, kz, ax, ay, az);
      const cx<TS> fnl = -((mul_i(m1, ax) + mul_i(m2, ay)) + mul_i(m3, az));
      rk.update(0, fnl, u0, r0, b.U + idx, b.R + idx, kk.ps.zero, kx, ky, kz);
    }
  }
}

// Incompressible (src_incompressible/mhdrhs.f90:117-232,468-518): group blockIdx.z = 0
// transforms the pressure flux and updates rho, rho u and p:
//   k.fp = (i k . fp_hat)/k^2, p_hat = -k.fp, fnl(rho u) = fp_hat + k.fp (i k)  (0 where k^2 < 1e-10)
// groups 1..3 advance Bx, By, Bz from the electric field as in the compressible pass.
template <class T, class TS, int NZ>
__global__ void __launch_bounds__(Col<T, NZ>::THREADS) k_passE3i(Bufs<T, TS> b, PassArgs a, PassK<T, TS> kk, const typename Store<T>::C* __restrict__ twz) {
  const PT<T>& pc = kk.pc;
  const KTab<T>& K = kk.K;
  using CL = Col<T, NZ>;
  using C = typename Store<T>::C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  if (a.st->halt) return;
  ColCtx<T, NZ, 3> x(reinterpret_cast<C*>(smem_raw));
  const Geo& g = a.g;
  const int grp = blockIdx.z;
  int kx = blockIdx.x * TX + x.c;
  int r = blockIdx.y * CL::NTILE + x.tl;
  bool ok = kx < g.kx_keep && r < g.nky();
  int ky = ok ? g.ky_of(r) : 0;
  long long col = (long long)ky * g.kxp + kx;
  long long zs = (long long)g.ny * g.kxp;
  const int sexp = -__ffs(NZ) + 1;
  // slots: 0..2 fp, 3 Ex, 4 Ey, 5 P7, 6 P5, 7 P6
  const int nin = grp == 0 ? 3 : (grp == 3 ? 1 : 2);
  const int ins[4][3] = {{0, 1, 2}, {6, 4, -1}, {7, 3, -1}, {5, -1, -1}};
#pragma unroll 1
  for (int k = 0; k < nin; k++) {
    const C* in = b.W2 + ins[grp][k] * g.fsc + col;
#pragma unroll
    for (int m = 0; m < CL::EPT; m++) {
      cx<T> w = ok ? Store<T>::ldg(in + x.j(m) * zs) : cx_zero<T>();
      Store<T>::stc(x.at(k, m), w);
    }
    __syncthreads();
    fft_lines<T, NZ, -1, TX, 1>(x.buf(k), x.c, x.t, true, twz, 1);
  }
  if (!ok) return;
  using CS = typename Store<TS>::C;
  const RkCtx<TS, T> rk = rk_ctx<T>(a, kk.ps, kk.KS);
  const T rr = Real<T>::from_d(a.st->r_ratio);
  // FP32 transforms with a wider state: FP32 increments and k^2 (RkCtx::update_f32)
  constexpr bool F32INC = std::is_same<T, float>::value && !std::is_same<TS, float>::value;
  const RkCtx<T, T> rkf = rk_ctx<T>(a, kk.pc, kk.K);
  const float ccf = a.st->f_cc[a.stage], ddcf = a.st->f_ddc[a.stage], itf = a.st->f_inv_tau;
  const float tsf = a.st->f_ts[a.stage];
#pragma unroll 1
  for (int m = 0; m < CL::EPT; m++) {
    int kz = x.j(m);
    if (!g.kz_in(kz)) continue;
    long long idx = kz * zs;
    auto val = [&](int bi) {
      cx<T> w = Store<T>::ldc(x.at(bi, m));
      return cx<T>{Real<T>::mul_pow2(w.re, sexp), Real<T>::mul_pow2(w.im, sexp)};
    };
    TS k2 = kk.ps.zero;
    T k2t;
    if constexpr (F32INC) {
      k2t = rkf.k2(kx, ky, kz);
    } else {
      k2 = rk.k2(kx, ky, kz);
      k2t = Cvt<T, TS>::r(k2);
    }
    // the update of variable v from its right-hand side fnl and its state value u
    auto upd = [&](int v, cx<T> fnl, cx<TS> u) {
      CS* U = b.U + v * g.fsc + col + idx;
      C* R = b.R + v * g.fsc + col + idx;
      if constexpr (F32INC) {
        const cx<float> r = a.stage > 0 ? Store<T>::ldc(R) : cx_zero<float>();
        rk.update_f32(v, fnl, u, r, U, R, k2t, kx, ky, kz, pc, ccf, ddcf, itf, tsf);
      } else {
        rk.update(v, cvtc<TS>(fnl), u, U, R, k2, kx, ky, kz);
      }
    };
    if (grp == 0) {
      T ax, ay, az;
      kfac(K, a.P, pc, rr, kx, ky, kz, ax, ay, az);
      cx<T> f0 = val(0), f1 = val(1), f2 = val(2);
      const bool small = Real<T>::lead(k2t) < 1e-10f;
      cx<T> kdot = cx_zero<T>();
      if (!small) {
        cx<T> sm = (mul_i(f0, ax) + mul_i(f1, ay)) + mul_i(f2, az);
        kdot = {sm.re / k2t, sm.im / k2t};
      }
      const cx<T> fm[3] = {small ? cx_zero<T>() : f0 + mul_i(kdot, ax), small ? cx_zero<T>() : f1 + mul_i(kdot, ay),
                           small ? cx_zero<T>() : f2 + mul_i(kdot, az)};
      for (int v = 0; v < 4; v++) upd(v, v == 0 ? cx_zero<T>() : fm[v - 1], Store<TS>::ldc(b.U + v * g.fsc + col + idx));
      // the new pressure replaces slot 8 before the update
      cx<TS> pn;
      if constexpr (F32INC) pn = IncCvt<TS>::from_f32(-kdot);
      else pn = cvtc<TS>(-kdot);
      upd(7, cx_zero<T>(), pn);
    } else {
      const int v = 3 + grp;
      cx<T> f = val(0);
      if (nin > 1) {
        cx<T> w = mul_i(val(1), K.kzd[kz]);
        f = v == 4 ? f + w : f - w;
      }
      upd(v, f, Store<TS>::ldc(b.U + v * g.fsc + col + idx));
    }
  }
}

}  // namespace laps
