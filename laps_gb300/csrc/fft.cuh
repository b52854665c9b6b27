// Batched 1-D complex FFTs of power-of-two length N held in shared memory.
//
// Algorithm: Stockham autosort (no bit reversal) with radix-16 stages and one final
// radix-2/4/8 stage, each thread owning 16 elements of a line per stage (N >= 16;
// a single radix-8 thread for N = 8).  For a stage of radix r after Ns points have been
// combined, butterfly b (0 <= b < N/r) reads x[b + i N/r], multiplies by w^(i k N/(Ns r))
// with k = b mod Ns, does an r-point DFT and writes y[(b / Ns) Ns r + k + i Ns].
// This replaces the reference's per-line FFTW plans (src_compressible/fftw.f90:27-33),
// which compute the same unnormalised DFT: sign -1 forward, +1 backward.
//
// Layout: element j of line `l` lives at s[j * JS + l * LS] (Store<T>::C units).  Column
// tiles use JS = TX, LS = 1 (a quarter-warp touches one 128-byte row: conflict-free);
// rows use JS = 1, LS = line pitch.
#pragma once
#include <type_traits>

#include "arith.cuh"

namespace laps {

// compile-time float-float split of a double constant
#define LAPS_KC(name, val)                         \
  constexpr double name##_d = (val);              \
  constexpr float name##_h = (float)(name##_d);   \
  constexpr float name##_l = (float)(name##_d - (double)name##_h)

template <class T> __device__ __forceinline__ T kc(double d, float h, float l);
template <> __device__ __forceinline__ double kc<double>(double d, float, float) { return d; }
template <> __device__ __forceinline__ dd kc<dd>(double, float h, float l) { return {h, l}; }
template <> __device__ __forceinline__ float kc<float>(double, float h, float) { return h; }

LAPS_KC(K_SQH, 0.70710678118654752440);   // sqrt(2)/2
LAPS_KC(K_C8, 0.92387953251128675613);    // cos(pi/8)
LAPS_KC(K_S8, 0.38268343236508977173);    // sin(pi/8)

// x * exp(DIR * i * theta) for theta = pi/4 (w8), given cos = sin = sqrt(2)/2
template <class T, int DIR> __device__ __forceinline__ cx<T> rot45(cx<T> x) {
  const T c = kc<T>(K_SQH_d, K_SQH_h, K_SQH_l);
#if LAPS_PACKED_DD
  // float-float: both components in one packed pass, (x -/+ i x) c, with the operations of
  // the scalar form in each lane
  if constexpr (std::is_same<T, dd>::value) return (x + (DIR < 0 ? times_mi(x) : times_i(x))) * c;
#endif
  // DIR=-1: (1 - i)/sqrt2 * (a + ib) = ((a + b) + i (b - a)) / sqrt2
  if (DIR < 0) return {(x.re + x.im) * c, (x.im - x.re) * c};
  return {(x.re - x.im) * c, (x.im + x.re) * c};
}
template <class T, int DIR> __device__ __forceinline__ cx<T> rot135(cx<T> x) {
  const T c = kc<T>(K_SQH_d, K_SQH_h, K_SQH_l);
#if LAPS_PACKED_DD
  if constexpr (std::is_same<T, dd>::value) return DIR < 0 ? times_mi(rot45<T, DIR>(x)) : times_i(rot45<T, DIR>(x));
#endif
  // DIR=-1: (-1 - i)/sqrt2 * (a + ib) = ((b - a) + i (-a - b)) / sqrt2
  if (DIR < 0) return {(x.im - x.re) * c, -((x.re + x.im) * c)};
  return {-((x.re + x.im) * c), (x.re - x.im) * c};
}
// x * (c + DIR*i*s) with constants c, s
template <class T, int DIR> __device__ __forceinline__ cx<T> rotcs(cx<T> x, T c, T s) {
#if LAPS_PACKED_DD
  if constexpr (std::is_same<T, dd>::value) return x * c + (DIR < 0 ? times_mi(x) : times_i(x)) * s;
#endif
  if (DIR < 0) return {x.re * c + x.im * s, x.im * c - x.re * s};
  return {x.re * c - x.im * s, x.im * c + x.re * s};
}
template <class T, int DIR> __device__ __forceinline__ cx<T> mul_dir_i(cx<T> x) {
  return DIR < 0 ? times_mi(x) : times_i(x);
}

template <class T, int DIR> __device__ __forceinline__ void dft2(cx<T>* v) {
  cx<T> a = v[0], b = v[1];
  v[0] = a + b;
  v[1] = a - b;
}
template <class T, int DIR> __device__ __forceinline__ void dft4(cx<T>& x0, cx<T>& x1, cx<T>& x2, cx<T>& x3) {
  cx<T> a = x0 + x2, b = x0 - x2, c = x1 + x3, d = mul_dir_i<T, DIR>(x1 - x3);
  x0 = a + c;
  x2 = a - c;
  x1 = b + d;
  x3 = b - d;
}
template <class T, int DIR> __device__ __forceinline__ void dft4v(cx<T>* v) { dft4<T, DIR>(v[0], v[1], v[2], v[3]); }
template <class T, int DIR> __device__ __forceinline__ void dft8(cx<T>* v) {
  // decimation in time: E = DFT4(x0,x2,x4,x6), O = DFT4(x1,x3,x5,x7)
  cx<T> e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
  cx<T> o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
  dft4<T, DIR>(e0, e1, e2, e3);
  dft4<T, DIR>(o0, o1, o2, o3);
  o1 = rot45<T, DIR>(o1);
  o2 = mul_dir_i<T, DIR>(o2);
  o3 = rot135<T, DIR>(o3);
  v[0] = e0 + o0; v[4] = e0 - o0;
  v[1] = e1 + o1; v[5] = e1 - o1;
  v[2] = e2 + o2; v[6] = e2 - o2;
  v[3] = e3 + o3; v[7] = e3 - o3;
}
template <class T, int DIR> __device__ __forceinline__ void dft16(cx<T>* v) {
  // four-step 4 x 4: n = n1 + 4 n2, k = k2 + 4 k1
  cx<T> y[16];
#pragma unroll
  for (int n1 = 0; n1 < 4; n1++) {
    cx<T> a = v[n1], b = v[n1 + 4], c = v[n1 + 8], d = v[n1 + 12];
    dft4<T, DIR>(a, b, c, d);
    y[n1 * 4 + 0] = a; y[n1 * 4 + 1] = b; y[n1 * 4 + 2] = c; y[n1 * 4 + 3] = d;
  }
  const T c8 = kc<T>(K_C8_d, K_C8_h, K_C8_l), s8 = kc<T>(K_S8_d, K_S8_h, K_S8_l);
  // twiddles w16^(n1 k2)
  y[1 * 4 + 1] = rotcs<T, DIR>(y[5], c8, s8);          // w^1
  y[1 * 4 + 2] = rot45<T, DIR>(y[6]);                  // w^2
  y[1 * 4 + 3] = rotcs<T, DIR>(y[7], s8, c8);          // w^3
  y[2 * 4 + 1] = rot45<T, DIR>(y[9]);                  // w^2
  y[2 * 4 + 2] = mul_dir_i<T, DIR>(y[10]);             // w^4
  y[2 * 4 + 3] = rot135<T, DIR>(y[11]);                // w^6
  y[3 * 4 + 1] = rotcs<T, DIR>(y[13], s8, c8);         // w^3
  y[3 * 4 + 2] = rot135<T, DIR>(y[14]);                // w^6
  y[3 * 4 + 3] = -rotcs<T, DIR>(y[15], c8, s8);       // w^9 = -w^1
#pragma unroll
  for (int k2 = 0; k2 < 4; k2++) {
    cx<T> a = y[0 * 4 + k2], b = y[1 * 4 + k2], c = y[2 * 4 + k2], d = y[3 * 4 + k2];
    dft4<T, DIR>(a, b, c, d);
    v[k2] = a; v[k2 + 4] = b; v[k2 + 8] = c; v[k2 + 12] = d;
  }
}
template <class T, int DIR, int R> __device__ __forceinline__ void dft_r(cx<T>* v) {
  if (R == 2) dft2<T, DIR>(v);
  else if (R == 4) dft4v<T, DIR>(v);
  else if (R == 8) dft8<T, DIR>(v);
  else dft16<T, DIR>(v);
}

// Stage plan for length N.
template <int N> struct Plan {
  static constexpr int EPT = N >= 16 ? 16 : N;               // elements per thread per stage
  static constexpr int TPL = N / EPT;                        // threads per line
  static constexpr int NS16 = N >= 16 ? (N >= 4096 ? 3 : N >= 256 ? 2 : 1) : 0;
  static constexpr int REST = N >= 16 ? N / (NS16 == 1 ? 16 : NS16 == 2 ? 256 : 4096) : N;
  static constexpr int NSTAGE = NS16 + (REST > 1 ? 1 : 0);
};

// twiddle w_N^m (DIR=-1: exp(-2 pi i m/N)), read from a table of exp(-2 pi i j/Ntab)
template <class T, int DIR>
__device__ __forceinline__ cx<T> twiddle(const typename Store<T>::C* __restrict__ tw, int idx) {
  cx<T> w = Store<T>::ldg(tw + idx);
  return DIR < 0 ? w : conj(w);
}

// Shared-memory position of element j of a line: columns use j*JS; rows (JS == 1) are
// padded by one element after every 16 so that the radix-16 write pattern (stride 16
// elements) spreads over all banks.
template <int JS> __device__ __forceinline__ int sm_idx(int j) { return JS == 1 ? j + (j >> 4) : j * JS; }
template <int N> struct RowLen { static constexpr int V = N + N / 16; };  // padded length of a row line

// Barrier of a stage: the whole block, or only the warp when every line's threads and shared
// memory belong to one warp (WL: row lines of at most 32 threads, laid out consecutively).
template <bool WL> __device__ __forceinline__ void stage_sync() {
  if (WL) __syncwarp();
  else __syncthreads();
}

// One Stockham stage of radix R after ns points have been combined (ns a power of two, 1
// for the first stage: no twiddles), for every line of the tile.  Thread t of line l;
// threads with active == false only join the two barriers.
template <class T, int N, int DIR, int R, int JS, int LS, bool WL = false>
__device__ __forceinline__ void fft_stage(typename Store<T>::C* s, int l, int t, bool active, int ns, int lns,
                                          const typename Store<T>::C* __restrict__ tw, int twstep) {
  using P = Plan<N>;
  constexpr int NB = P::EPT / R;  // butterflies per thread
  cx<T> v[NB][R];
  typename Store<T>::C* line = s + l * LS;
  if (active) {
#pragma unroll
    for (int q = 0; q < NB; q++) {
      int b = t + q * P::TPL;
#pragma unroll
      for (int i = 0; i < R; i++) v[q][i] = Store<T>::ldc(line + sm_idx<JS>(b + i * (N / R)));
      if (ns > 1) {
        int k = b & (ns - 1);
        int step = (k * (N / R) >> lns) * twstep;  // k * N / (ns R)
#pragma unroll
        for (int i = 1; i < R; i++) v[q][i] = v[q][i] * twiddle<T, DIR>(tw, i * step);
      }
    }
  }
  stage_sync<WL>();
  if (active) {
#pragma unroll
    for (int q = 0; q < NB; q++) {
      int b = t + q * P::TPL;
      int k = b & (ns - 1);
      dft_r<T, DIR, R>(v[q]);
      int base = ((b >> lns) << lns) * R + k;
#pragma unroll
      for (int i = 0; i < R; i++) Store<T>::stc(line + sm_idx<JS>(base + i * ns), v[q][i]);
    }
  }
  stage_sync<WL>();
}

// Full FFT of every line of the tile (unnormalised).  Every thread of the block (WL: of the
// warp) calls it.  The radix-16 stages run in a rolled loop (one copy of their code); the last
// radix-2/4/8 stage follows.  tw: table of exp(-2 pi i j / (N*twstep)), j = 0..N*twstep-1.
template <class T, int N, int DIR, int JS, int LS, bool WL = false>
__device__ __forceinline__ void fft_lines(typename Store<T>::C* s, int l, int t, bool active,
                                          const typename Store<T>::C* __restrict__ tw, int twstep) {
  using P = Plan<N>;
  static_assert(!WL || (JS == 1 && P::TPL <= 32), "warp-local lines are rows of at most one warp");
  if constexpr (N == 1) {  // a length-1 transform is the identity (nz = 1)
    stage_sync<WL>();
  } else if constexpr (N < 16) {
    fft_stage<T, N, DIR, N, JS, LS, WL>(s, l, t, active, 1, 0, tw, twstep);
  } else {
    int ns = 1, lns = 0;
#pragma unroll 1
    for (int st = 0; st < P::NS16; st++) {
      fft_stage<T, N, DIR, 16, JS, LS, WL>(s, l, t, active, ns, lns, tw, twstep);
      ns <<= 4;
      lns += 4;
    }
    if constexpr (P::REST > 1) fft_stage<T, N, DIR, P::REST, JS, LS, WL>(s, l, t, active, ns, lns, tw, twstep);
  }
}

// Forward transform of one warp-local row of N points as a real call (not inlined), so that
// callers transforming in both directions carry one copy of the butterflies: the backward
// transform is conj(forward(conj(x))).  For float-float rows, whose code otherwise outgrows the
// instruction cache (the x pass stalled on instruction fetch first).
template <class T, int N>
__device__ __noinline__ void fft_row_fwd_call(typename Store<T>::C* z, int t, bool active,
                                              const typename Store<T>::C* __restrict__ tw, int twstep) {
  fft_lines<T, N, -1, 1, 0, true>(z, 0, t, active, tw, twstep);
}
// Conjugate the elements t + 16 i (i < 16) of a 256-point row: the elements thread t loads
// first and stores last in fft_lines (two radix-16 stages), so no barrier is needed around it
template <class T>
__device__ __forceinline__ void row256_conj(typename Store<T>::C* z, int t, bool active) {
  if (!active) return;
#pragma unroll
  for (int i = 0; i < 16; i++) {
    typename Store<T>::C* p = z + sm_idx<1>(t + 16 * i);
    cx<T> v = Store<T>::ldc(p);
    Store<T>::stc(p, cx<T>{v.re, -v.im});
  }
}
template <class T, int N, int DIR>
__device__ __forceinline__ void fft_row_shared(typename Store<T>::C* z, int t, bool active,
                                               const typename Store<T>::C* __restrict__ tw, int twstep) {
  static_assert(N == 256, "the conjugation pattern is that of two radix-16 stages");
  if (DIR > 0) row256_conj<T>(z, t, active);
  fft_row_fwd_call<T, N>(z, t, active, tw, twstep);
  if (DIR > 0) row256_conj<T>(z, t, active);
}

// Two tiles transformed together (column passes with two inputs): one pass over the stages,
// the same twiddles applied to both, half the barriers.  FP32 lines only (two 16-element
// sets of float-float or FP64 values would not fit the register budget); other types
// transform the two buffers one after the other.
template <class T, int N, int DIR, int R, int JS>
__device__ __forceinline__ void fft_stage2(typename Store<T>::C* s0, typename Store<T>::C* s1, int l, int t, int ns, int lns,
                                           const typename Store<T>::C* __restrict__ tw, int twstep) {
  using P = Plan<N>;
  constexpr int NB = P::EPT / R;
  cx<T> v[2][NB][R];
  typename Store<T>::C* line0 = s0 + l;
  typename Store<T>::C* line1 = s1 + l;
#pragma unroll
  for (int q = 0; q < NB; q++) {
    int b = t + q * P::TPL;
#pragma unroll
    for (int i = 0; i < R; i++) {
      v[0][q][i] = Store<T>::ldc(line0 + sm_idx<JS>(b + i * (N / R)));
      v[1][q][i] = Store<T>::ldc(line1 + sm_idx<JS>(b + i * (N / R)));
    }
    if (ns > 1) {
      int k = b & (ns - 1);
      int step = (k * (N / R) >> lns) * twstep;
#pragma unroll
      for (int i = 1; i < R; i++) {
        const cx<T> w = twiddle<T, DIR>(tw, i * step);
        v[0][q][i] = v[0][q][i] * w;
        v[1][q][i] = v[1][q][i] * w;
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < NB; q++) {
    int b = t + q * P::TPL;
    int k = b & (ns - 1);
    dft_r<T, DIR, R>(v[0][q]);
    dft_r<T, DIR, R>(v[1][q]);
    int base = ((b >> lns) << lns) * R + k;
#pragma unroll
    for (int i = 0; i < R; i++) {
      Store<T>::stc(line0 + sm_idx<JS>(base + i * ns), v[0][q][i]);
      Store<T>::stc(line1 + sm_idx<JS>(base + i * ns), v[1][q][i]);
    }
  }
  __syncthreads();
}

// FFT of the column tiles s0 and, when `both`, s1 (block-uniform); every thread calls it
template <class T, int N, int DIR, int JS, int LS>
__device__ __forceinline__ void fft_lines_pair(typename Store<T>::C* s0, typename Store<T>::C* s1, bool both, int l, int t,
                                               const typename Store<T>::C* __restrict__ tw, int twstep) {
  using P = Plan<N>;
  constexpr bool PAIR = sizeof(typename Store<T>::C) == 8 && N >= 16 && LS == 1;
  if constexpr (PAIR) {
    if (both) {
      int ns = 1, lns = 0;
#pragma unroll 1
      for (int st = 0; st < P::NS16; st++) {
        fft_stage2<T, N, DIR, 16, JS>(s0, s1, l, t, ns, lns, tw, twstep);
        ns <<= 4;
        lns += 4;
      }
      if constexpr (P::REST > 1) fft_stage2<T, N, DIR, P::REST, JS>(s0, s1, l, t, ns, lns, tw, twstep);
      return;
    }
  }
  fft_lines<T, N, DIR, JS, LS>(s0, l, t, true, tw, twstep);
  if (both) fft_lines<T, N, DIR, JS, LS>(s1, l, t, true, tw, twstep);
}

}  // namespace laps
