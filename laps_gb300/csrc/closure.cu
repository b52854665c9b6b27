// Learned subgrid closure: 3x3x3 periodic convolutions in BF16 on the tensor cores.
//
// The closure net (4 layers of 3x3x3 convolutions, 32 channels, GELU) maps the box-filtered
// coarse velocity and magnetic field to subgrid stresses.  Each layer is an implicit GEMM
//   out[v][co] = sum_{tap, ci} in[v + shift(tap)][ci] * W[tap][co][ci]
// with M = voxels (a tile is 128 consecutive voxels of one x row), N = output channels and
// K = 27 taps x input channels, issued as tcgen05.mma (kind::f16, BF16 operands, FP32
// accumulator in tensor memory).
//
// Activation layout (every layer's input and output): channels-last BF16 with a one-voxel
// periodic halo on x, element (z, y, xp, c) at ((z * ny + y) * (nx + 2) + xp) * C + c, xp =
// x + 1, xp = 0 and nx + 1 holding x = nx - 1 and x = 0.  A tap is then a shift of the row
// index only: the tensor map is 2-D {C channels, nz * ny * (nx + 2) rows}, and every TMA box
// {8 channels, 128 rows} starts at channel 0, 8, 16 or 24 (16-byte aligned) - y and z wrap
// by choosing the source row, x by the halo.  C (the padded channel count) is 16 or 32.
//
// Shared memory holds all 27 taps of the packed weights for the whole kernel and a ring of
// activation stages, one per (dz, dy): the 130 voxels x0 - 1 .. x0 + 128 of the source row,
// which serve the three dx taps.  Operand layout in shared memory (no swizzle, K-major): core
// matrices of 8 rows x 16 bytes stored contiguously and one after the other along M, so every
// row lies 16 bytes after the previous one and the operand of tap dx is the same stage with
// its start moved by dx rows; chunk k of 8 channels is one TMA box of 130 rows (2080 B) at a
// 2176-byte stride (TMA destinations sit on 128-byte boundaries), so core matrices adjacent in
// M are 128 B apart and those adjacent in K 2176 B apart.  The packed
// weights of a tap are [K chunk][N rows][8], N-adjacent 128 B apart, K-adjacent N * 16 B apart.
//
// Roles (192 threads, persistent over tiles): warp 0 issues the TMA loads, warp 1 allocates
// tensor memory and issues the MMAs, warps 2-5 read the accumulator back (tcgen05.ld; warp w
// may read TMEM lanes 32 (w % 4) .. +31) and run the epilogue.  Two accumulators alternate so
// that a tile's epilogue overlaps the next tile's MMAs.  Every mbarrier wait is bounded by
// time (2 s on the global timer): a wait that runs out sets the error word and the block
// leaves its loops, waits (bounded) for its own copies and MMAs, frees its tensor memory and
// returns.
//
// No counterpart in the reference: the closure is an addition to the solver.
#include <cuda_bf16.h>
#include <string>
#include "launch.cuh"
#include "tma.cuh"

namespace laps {

constexpr int CONV_TILE = 128;     // voxels per tile (MMA M)
#ifndef LAPS_CONV_STAGES
#define LAPS_CONV_STAGES 6
#endif
constexpr int CONV_STAGES = LAPS_CONV_STAGES;  // activation stages in flight
constexpr int CONV_THREADS = 192;  // producer warp, MMA warp, 4 epilogue warps
#ifndef LAPS_WGRAD_SWAP
#define LAPS_WGRAD_SWAP false
#endif

struct ConvArgs {
  int nx, ny, nz, ntiles;
  int act;                      // 0 linear, 1 GELU (keeps the pre-activation), 2 gradient gate
  const float* bias;            // [N] (zero past the layer's own channels) or null
  const __nv_bfloat16* gate;    // act 2: pre-activation z of the layer whose output is the input
  __nv_bfloat16* y;             // output, padded layout, N channels
  __nv_bfloat16* zpre;          // act 1: pre-activation (padded layout) or null
  int* err;                     // error word: 1 = a bounded wait ran out
};

__device__ __forceinline__ uint64_t gtime_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}
// bounded wait on an mbarrier phase: false after 2 s
__device__ __forceinline__ bool conv_wait(uint64_t* bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = gtime_ns();
  while (!mbar_try_wait(bar, parity))
    if (gtime_ns() - t0 > 2000000000ull) return false;
  return true;
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// shared-memory matrix descriptor: no swizzle, start / leading (K) / stride (M or N) byte offsets
__device__ __forceinline__ uint64_t smem_desc(const void* p, uint32_t lbo, uint32_t sbo) {
  const uint32_t a = smem_u32(p);
  return (uint64_t)((a & 0x3FFFF) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) | (1ull << 46);
}
// instruction descriptor of kind::f16: BF16 A and B (K-major), FP32 D, M = 128, N = n
__host__ __device__ constexpr uint32_t mma_idesc_bf16(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(CONV_TILE >> 4) << 24);
}
__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}
// the mbarrier gets one arrival when every MMA this thread issued before has completed
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// 32 lanes x N columns of 32-bit accumulator -> registers (thread i of the warp: lane base + i)
template <int N> __device__ __forceinline__ void tmem_load(uint32_t taddr, float* v) {
  uint32_t r[N];
  if constexpr (N == 32) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
  } else {
    static_assert(N == 16, "16 or 32 output channels");
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
        "[%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
  }
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < N; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float z) {
  return 0.5f * (1.0f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * __expf(-0.5f * z * z);
}

template <int KC, int NP> struct ConvCfg {
  static constexpr int A_ROWS = CONV_TILE + 2;                // x0 - 1 .. x0 + 128: the three dx taps
  static constexpr int A_BOX = A_ROWS * 16;                   // 8 channels of those voxels (one TMA box)
  // chunk stride: a TMA destination in shared memory must be 128-byte aligned
  static constexpr int A_CHUNK = (A_BOX + 127) / 128 * 128;
  static constexpr int A_BYTES = KC * A_CHUNK;                // one (dz, dy) stage
  static_assert(A_CHUNK % 128 == 0 && A_BYTES % 128 == 0, "TMA destinations on 128-byte boundaries");
  static constexpr int B_TAP = KC * NP * 16;                  // one tap of packed weights
  static constexpr int B_BYTES = 27 * B_TAP;
  // an operand read with its two strides exchanged would reach 16 x 2 KB past a stage's start:
  // the region after the last stage is at least that long, so such reads stay in the block
  // (and the weights read that way reach < 4 KB past their end)
  static constexpr int TAIL = B_BYTES + 4096 > 33 * 1024 ? B_BYTES + 4096 : 33 * 1024;
  static constexpr int SMEM = 1024 + CONV_STAGES * A_BYTES + TAIL + NP * 4;
  static constexpr int TMEM_COLS = 2 * NP < 32 ? 32 : 2 * NP;
};

template <int KC, int NP>
__global__ void __launch_bounds__(CONV_THREADS, 1)
    k_conv3(const __grid_constant__ CUtensorMap tx, const uint4* __restrict__ wpk, ConvArgs a) {
  using CF = ConvCfg<KC, NP>;
  extern __shared__ unsigned char smem_conv[];
  __shared__ __align__(8) uint64_t full[CONV_STAGES], empty[CONV_STAGES], accf[2], acce[2], drain;
  __shared__ uint32_t tmem_base_sh;
  __shared__ volatile int bail;  // set by a role whose wait ran out; the others leave their loops
  unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_conv) + 1023) & ~uintptr_t(1023));
  unsigned char* A = sm;
  unsigned char* B = sm + CONV_STAGES * CF::A_BYTES;
  float* bias_s = reinterpret_cast<float*>(B + CF::TAIL);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  // the packed weights and the bias into shared memory, visible to the tensor core's proxy
  for (int i = threadIdx.x; i < CF::B_BYTES / 16; i += CONV_THREADS) reinterpret_cast<uint4*>(B)[i] = wpk[i];
  for (int i = threadIdx.x; i < NP; i += CONV_THREADS) bias_s[i] = a.bias ? a.bias[i] : 0.0f;
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  if (threadIdx.x == 0) {
    for (int s = 0; s < CONV_STAGES; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int i = 0; i < 2; i++) {
      mbar_init(&accf[i], 1);
      mbar_init(&acce[i], 4 * 32);
    }
    mbar_init(&drain, 1);
    mbar_fence_init();
    bail = 0;
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_sh)),
                 "r"((uint32_t)CF::TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = tmem_base_sh;
  const int xt = a.nx / CONV_TILE;
  const int pitch = a.nx + 2;

  if (warp == 0) {
    // ------------------------------------------------------------ producer: one tap per stage
    if (lane == 0) {
      int s = 0;
      uint32_t ph = 0;
      uint32_t issued = 0, last_ph = 0;  // stages filled at least once; parity of each stage's last fill
      for (int tile = blockIdx.x; tile < a.ntiles && !bail; tile += gridDim.x) {
        const int x0 = (tile % xt) * CONV_TILE;
        const int r = tile / xt, y = r % a.ny, z = r / a.ny;
        for (int t = 0; t < 9; t++) {  // one stage per (dz, dy): the rows of all three dx taps
          if (!conv_wait(&empty[s], ph ^ 1u)) {
            bail = 1;
            atomicExch(a.err, 1);
            break;
          }
          const int dz = t / 3, dy = t % 3;
          const int zz = (z + dz - 1 + a.nz) % a.nz, yy = (y + dy - 1 + a.ny) % a.ny;
          const int row = (zz * a.ny + yy) * pitch + x0;
          // (a destination off its 128-byte boundary is not loaded: the error word is set and
          // the wait on this stage runs out instead of the copy faulting)
          const bool aligned = (smem_u32(A + s * CF::A_BYTES) & 127u) == 0;
          if (!aligned) {
            atomicExch(a.err, 2);
            bail = 1;
            break;
          }
          mbar_arrive_expect_tx(&full[s], KC * CF::A_BOX);
#pragma unroll
          for (int k = 0; k < KC; k++) tma_load_2d(A + s * CF::A_BYTES + k * CF::A_CHUNK, &tx, k * 8, row, &full[s]);
          issued |= 1u << s;
          last_ph = (last_ph & ~(1u << s)) | (ph << s);
          if (++s == CONV_STAGES) {
            s = 0;
            ph ^= 1u;
          }
        }
      }
      // every copy this thread issued has landed before the block can leave
      for (int i = 0; i < CONV_STAGES; i++)
        if (issued >> i & 1u) conv_wait(&full[i], last_ph >> i & 1u);
    }
  } else if (warp == 1) {
    // ------------------------------------------------------------ MMA issuer
    if (lane == 0) {
      constexpr uint32_t IDESC = mma_idesc_bf16(NP);
      int s = 0, acc = 0;
      uint32_t ph = 0, aph = 0;
      for (int tile = blockIdx.x; tile < a.ntiles && !bail; tile += gridDim.x) {
        if (!conv_wait(&acce[acc], aph ^ 1u)) {
          bail = 1;
          atomicExch(a.err, 1);
          break;
        }
        tc_fence_after();
        const uint32_t d = tbase + acc * NP;
        bool ok = true;
        for (int t = 0; t < 9; t++) {
          if (!conv_wait(&full[s], ph)) {
            ok = false;
            break;
          }
          tc_fence_after();
          // rows lie 16 bytes apart (core matrices of 8 rows are contiguous), so the operand of
          // tap dx starts dx rows into the stage
#pragma unroll
          for (int dx = 0; dx < 3; dx++)
#pragma unroll
            for (int j = 0; j < KC / 2; j++) {
              const uint64_t ad = smem_desc(A + s * CF::A_BYTES + 2 * j * CF::A_CHUNK + dx * 16, CF::A_CHUNK, 128);
              const uint64_t bd = smem_desc(B + (3 * t + dx) * CF::B_TAP + 2 * j * NP * 16, NP * 16, 128);
              umma_bf16(d, ad, bd, IDESC, (t | dx | j) != 0);
            }
          umma_commit(&empty[s]);  // the stage is free once these MMAs have read it
          if (++s == CONV_STAGES) {
            s = 0;
            ph ^= 1u;
          }
        }
        if (!ok) {
          bail = 1;
          atomicExch(a.err, 1);
          break;
        }
        umma_commit(&accf[acc]);
        acc ^= 1;
        if (acc == 0) aph ^= 1u;
      }
      // every MMA this thread issued has completed before the tensor memory is freed
      umma_commit(&drain);
      conv_wait(&drain, 0);
    }
  } else {
    // ------------------------------------------------------------ epilogue: 4 warps, 128 voxels
    const int q = warp & 3;  // TMEM lane quarter this warp may read
    const int row = q * 32 + lane;
    int acc = 0;
    uint32_t aph = 0;
    // (tcgen05.ld is warp-collective: the loop exit and the wait's outcome are made uniform
    // over the warp)
    for (int tile = blockIdx.x; tile < a.ntiles; tile += gridDim.x) {
      if (__any_sync(0xffffffffu, bail != 0)) break;
      if (!__all_sync(0xffffffffu, conv_wait(&accf[acc], aph))) {
        if (lane == 0) {
          bail = 1;
          atomicExch(a.err, 1);
        }
        break;
      }
      tc_fence_after();
      float v[NP];
      tmem_load<NP>(tbase + ((uint32_t)(q * 32) << 16) + acc * NP, v);
      tc_fence_before();
      mbar_arrive(&acce[acc]);
      acc ^= 1;
      if (acc == 0) aph ^= 1u;
      const int x0 = (tile % xt) * CONV_TILE;
      const int r = tile / xt, y = r % a.ny, z = r / a.ny;
      const int x = x0 + row;
      const long long vrow = (long long)(z * a.ny + y) * pitch;
      const long long vo = (vrow + x + 1) * NP;
      __align__(16) __nv_bfloat16 out[NP], zp[NP];
      if (a.act == 2) {
        const uint4* g = reinterpret_cast<const uint4*>(a.gate + vo);
        __align__(16) __nv_bfloat16 gz[NP];
#pragma unroll
        for (int i = 0; i < NP / 8; i++) reinterpret_cast<uint4*>(gz)[i] = g[i];
#pragma unroll
        for (int c = 0; c < NP; c++) out[c] = __float2bfloat16_rn(v[c] * gelu_grad(__bfloat162float(gz[c])));
      } else {
#pragma unroll
        for (int c = 0; c < NP; c++) {
          const float zz = v[c] + bias_s[c];
          zp[c] = __float2bfloat16_rn(zz);
          out[c] = __float2bfloat16_rn(a.act == 1 ? gelu(zz) : zz);
        }
      }
      uint4* yo = reinterpret_cast<uint4*>(a.y + vo);
#pragma unroll
      for (int i = 0; i < NP / 8; i++) yo[i] = reinterpret_cast<const uint4*>(out)[i];
      // the periodic x halo of the output
      if (x == 0 || x == a.nx - 1) {
        uint4* yh = reinterpret_cast<uint4*>(a.y + (vrow + (x == 0 ? a.nx + 1 : 0)) * NP);
#pragma unroll
        for (int i = 0; i < NP / 8; i++) yh[i] = reinterpret_cast<const uint4*>(out)[i];
      }
      if (a.act == 1 && a.zpre) {
        uint4* zo = reinterpret_cast<uint4*>(a.zpre + vo);
#pragma unroll
        for (int i = 0; i < NP / 8; i++) zo[i] = reinterpret_cast<const uint4*>(zp)[i];
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"((uint32_t)CF::TMEM_COLS)
                 : "memory");
  }
}

// ---------------------------------------------------------------------------- weight gradient
// dW[t][co][ci] = sum_v dZ[v][co] * X[v + shift(t)][ci]: an MMA with K = voxels.  M = TG taps x
// CI input channels = 128 rows (TG = 128 / CI), N = NP output channels; both operands are
// MN-major (channels contiguous in memory): a stage holds KV = 64 voxels, one 1 KB TMA box
// {8 channels, 64 voxels} per 8 rows of M or N (core matrices of 8 voxels x 16 B, adjacent in
// K 128 B apart, adjacent in M or N 1 KB apart).  Grid: tap groups x voxel splits; each block
// accumulates its voxel range in tensor memory and adds its 128 x NP partial sums to dW (FP32,
// zeroed by the entry point) with atomics.
constexpr int WG_KV = 64;
constexpr int WG_STAGES = 4;

template <int CI, int NP> struct WgCfg {
  static constexpr int TG = 128 / CI;                    // taps per block
  static constexpr int GROUPS = (27 + TG - 1) / TG;      // tap groups
  static constexpr int BOX = WG_KV * 16;                 // one box: 8 channels x 64 voxels
  static constexpr int A_BYTES = 16 * BOX;               // 128 rows of M
  static constexpr int B_BYTES = (NP / 8) * BOX;
  static constexpr int STAGE = A_BYTES + B_BYTES;
  static constexpr int SMEM = 1024 + WG_STAGES * STAGE + 4096;
};

template <int CI, int NP, bool SWAP>
__global__ void __launch_bounds__(CONV_THREADS, 1)
    k_conv3_wgrad(const __grid_constant__ CUtensorMap tx, const __grid_constant__ CUtensorMap tz, float* __restrict__ dw,
                  int nx, int ny, int nz, int nchunks, int* err) {
  using CF = WgCfg<CI, NP>;
  extern __shared__ unsigned char smem_wg[];
  __shared__ __align__(8) uint64_t full[WG_STAGES], empty[WG_STAGES], accf, drain;
  __shared__ uint32_t tmem_base_sh;
  __shared__ volatile int bail;
  unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_wg) + 1023) & ~uintptr_t(1023));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int group = blockIdx.x;
  if (threadIdx.x == 0) {
    for (int s = 0; s < WG_STAGES; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(&accf, 1);
    mbar_init(&drain, 1);
    mbar_fence_init();
    bail = 0;
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_sh)), "r"(32u)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = tmem_base_sh;
  const int xb = nx / WG_KV, pitch = nx + 2;
  // the chunks of this block: c = blockIdx.y, blockIdx.y + gridDim.y, ...
  const int my = blockIdx.y < nchunks ? (nchunks - 1 - blockIdx.y) / gridDim.y + 1 : 0;
  // taps of this group that exist (the last group may be short); rows of missing taps are
  // never loaded and their sums never stored
  const int ntap = 27 - group * CF::TG < CF::TG ? 27 - group * CF::TG : CF::TG;
  const uint32_t stage_tx = (uint32_t)(ntap * (CI / 8) * CF::BOX + CF::B_BYTES);

  if (warp == 0) {
    if (lane == 0) {
      int s = 0;
      uint32_t ph = 0, issued = 0, last_ph = 0;
      for (int i = 0; i < my && !bail; i++) {
        const int c = blockIdx.y + i * gridDim.y;
        const int x0 = (c % xb) * WG_KV;
        const int r = c / xb, y = r % ny, z = r / ny;
        if (!conv_wait(&empty[s], ph ^ 1u)) {
          bail = 1;
          atomicExch(err, 1);
          break;
        }
        mbar_arrive_expect_tx(&full[s], stage_tx);
        unsigned char* st = sm + s * CF::STAGE;
        for (int tl = 0; tl < ntap; tl++) {
          const int t = group * CF::TG + tl;
          const int dz = t / 9, dy = (t / 3) % 3, dx = t % 3;
          const int zz = (z + dz - 1 + nz) % nz, yy = (y + dy - 1 + ny) % ny;
          const int row = (zz * ny + yy) * pitch + x0 + dx;
          for (int k = 0; k < CI / 8; k++) tma_load_2d(st + (tl * (CI / 8) + k) * CF::BOX, &tx, k * 8, row, &full[s]);
        }
        const int rowz = (z * ny + y) * pitch + x0 + 1;
        for (int k = 0; k < NP / 8; k++) tma_load_2d(st + CF::A_BYTES + k * CF::BOX, &tz, k * 8, rowz, &full[s]);
        issued |= 1u << s;
        last_ph = (last_ph & ~(1u << s)) | (ph << s);
        if (++s == WG_STAGES) {
          s = 0;
          ph ^= 1u;
        }
      }
      for (int i = 0; i < WG_STAGES; i++)
        if (issued >> i & 1u) conv_wait(&full[i], last_ph >> i & 1u);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // kind::f16, BF16 A and B, both MN-major, FP32 D, M = 128, N = NP
      constexpr uint32_t IDESC = mma_idesc_bf16(NP) | (1u << 15) | (1u << 16);
      // no swizzle: leading byte offset = between core matrices adjacent in K, stride byte
      // offset = between those adjacent in M / N (SWAP exchanges the two)
      constexpr uint32_t LBO = SWAP ? CF::BOX : 128, SBO = SWAP ? 128 : CF::BOX;
      int s = 0;
      uint32_t ph = 0;
      bool ok = true;
      for (int i = 0; i < my && !bail; i++) {
        if (!conv_wait(&full[s], ph)) {
          ok = false;
          break;
        }
        tc_fence_after();
        unsigned char* st = sm + s * CF::STAGE;
#pragma unroll
        for (int kk = 0; kk < WG_KV / 16; kk++) {  // 16 voxels per MMA: two core matrices along K
          const uint64_t ad = smem_desc(st + kk * 256, LBO, SBO);
          const uint64_t bd = smem_desc(st + CF::A_BYTES + kk * 256, LBO, SBO);
          umma_bf16(tbase, ad, bd, IDESC, (i | kk) != 0);
        }
        umma_commit(&empty[s]);
        if (++s == WG_STAGES) {
          s = 0;
          ph ^= 1u;
        }
      }
      if (!ok) {
        bail = 1;
        atomicExch(err, 1);
      } else if (my > 0) {
        umma_commit(&accf);
      }
      umma_commit(&drain);
      conv_wait(&drain, 0);
    }
  } else if (my > 0) {
    const int q = warp & 3;
    const int row = q * 32 + lane;  // M row = (tap in group, input channel)
    bool ok = __all_sync(0xffffffffu, conv_wait(&accf, 0));
    if (ok && !__any_sync(0xffffffffu, bail != 0)) {
      tc_fence_after();
      float v[NP];
      tmem_load<NP>(tbase + ((uint32_t)(q * 32) << 16), v);
      tc_fence_before();
      const int tl = row / CI, ci = row % CI;
      const int t = group * CF::TG + tl;
      if (t < 27) {
#pragma unroll
        for (int co = 0; co < NP; co++) atomicAdd(&dw[((long long)t * NP + co) * CI + ci], v[co]);
      }
    } else if (!ok && lane == 0) {
      bail = 1;
      atomicExch(err, 1);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(32u) : "memory");
  }
}

// ---------------------------------------------------------------------------- closure data
// Subgrid quantities of the incompressible run: a box filter of width r (fine n_f = r n_c)
// followed by sampling on the coarse grid.  Per coarse voxel, with u = (rho u) / rho and b = B:
//   coarse state  (rho, rho u, B, p) box means (reference order, 8 fields)
//   targets 0..5  tau_ij = <u_i u_j> - <u_i><u_j> - (<b_i b_j> - <b_i><b_j>), ij = xx xy xz yy yz zz
//                 (the symmetric Reynolds-minus-Maxwell stress the coarse momentum misses)
//   targets 6..8  eps = <u x b> - <u> x <b> (the subgrid electromotive force)
//   targets 9..11 the Hall part of the subgrid electromotive force: zero (the runs this
//                 filter serves have d_i = 0)
__global__ void k_closure_filter(const double* __restrict__ fine, int nf, int r, double* __restrict__ coarse,
                                 float* __restrict__ tgt) {
  const int nc = nf / r;
  const long long ncell = (long long)nc * nc * nc, nfp = (long long)nf * nf * nf;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < ncell; c += (long long)gridDim.x * blockDim.x) {
    const int cx = (int)(c % nc), cy = (int)((c / nc) % nc), cz = (int)(c / ((long long)nc * nc));
    double m[8] = {0, 0, 0, 0, 0, 0, 0, 0};  // means of the 8 state fields
    double su[3] = {0, 0, 0}, sb[3] = {0, 0, 0}, uu[6] = {0, 0, 0, 0, 0, 0}, bb[6] = {0, 0, 0, 0, 0, 0}, ub[3] = {0, 0, 0};
    for (int dz = 0; dz < r; dz++)
      for (int dy = 0; dy < r; dy++)
        for (int dx = 0; dx < r; dx++) {
          const long long i = ((long long)(cz * r + dz) * nf + (cy * r + dy)) * nf + (cx * r + dx);
          double q[8];
#pragma unroll
          for (int f = 0; f < 8; f++) {
            q[f] = fine[f * nfp + i];
            m[f] += q[f];
          }
          const double u[3] = {q[1] / q[0], q[2] / q[0], q[3] / q[0]}, b[3] = {q[4], q[5], q[6]};
          int k = 0;
#pragma unroll
          for (int a = 0; a < 3; a++) {
            su[a] += u[a];
            sb[a] += b[a];
#pragma unroll
            for (int e = a; e < 3; e++, k++) {
              uu[k] += u[a] * u[e];
              bb[k] += b[a] * b[e];
            }
          }
          ub[0] += u[1] * b[2] - u[2] * b[1];
          ub[1] += u[2] * b[0] - u[0] * b[2];
          ub[2] += u[0] * b[1] - u[1] * b[0];
        }
    const double w = 1.0 / ((double)r * r * r);
#pragma unroll
    for (int f = 0; f < 8; f++) coarse[f * ncell + c] = m[f] * w;
    double ua[3], ba[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
      ua[a] = su[a] * w;
      ba[a] = sb[a] * w;
    }
    int k = 0;
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
      for (int e = a; e < 3; e++, k++)
        tgt[k * ncell + c] = (float)((uu[k] * w - ua[a] * ua[e]) - (bb[k] * w - ba[a] * ba[e]));
    tgt[6 * ncell + c] = (float)(ub[0] * w - (ua[1] * ba[2] - ua[2] * ba[1]));
    tgt[7 * ncell + c] = (float)(ub[1] * w - (ua[2] * ba[0] - ua[0] * ba[2]));
    tgt[8 * ncell + c] = (float)(ub[2] * w - (ua[0] * ba[1] - ua[1] * ba[0]));
    for (int f = 9; f < 12; f++) tgt[f * ncell + c] = 0.0f;
  }
}

// the net's input from a coarse state (8 fields): u = (rho u) / rho and B, divided by su and
// sb, in the convolutions' padded layout (16 channels, 6 used, x halo)
__global__ void k_closure_pack_input(const double* __restrict__ st, __nv_bfloat16* __restrict__ x, int n, double su, double sb) {
  const long long np = (long long)n * n * n;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < np; i += (long long)gridDim.x * blockDim.x) {
    const int ix = (int)(i % n);
    const long long row = i / n;
    const double rho = st[i];
    __align__(16) __nv_bfloat16 v[16];
#pragma unroll
    for (int c = 0; c < 16; c++) v[c] = __float2bfloat16_rn(0.0f);
#pragma unroll
    for (int a = 0; a < 3; a++) {
      v[a] = __float2bfloat16_rn((float)(st[(1 + a) * np + i] / rho / su));
      v[3 + a] = __float2bfloat16_rn((float)(st[(4 + a) * np + i] / sb));
    }
    const long long o = (row * (n + 2) + ix + 1) * 16;
    reinterpret_cast<uint4*>(x + o)[0] = reinterpret_cast<const uint4*>(v)[0];
    reinterpret_cast<uint4*>(x + o)[1] = reinterpret_cast<const uint4*>(v)[1];
    if (ix == 0 || ix == n - 1) {
      const long long h = (row * (n + 2) + (ix == 0 ? n + 1 : 0)) * 16;
      reinterpret_cast<uint4*>(x + h)[0] = reinterpret_cast<const uint4*>(v)[0];
      reinterpret_cast<uint4*>(x + h)[1] = reinterpret_cast<const uint4*>(v)[1];
    }
  }
}

// the net's output (padded layout, 16 channels, 12 used) times s -> 12 real FP64 fields
__global__ void k_closure_unpack(const __nv_bfloat16* __restrict__ y, double* __restrict__ tau, int n, double s) {
  const long long np = (long long)n * n * n;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < np; i += (long long)gridDim.x * blockDim.x) {
    const long long o = ((i / n) * (n + 2) + i % n + 1) * 16;
    __align__(16) __nv_bfloat16 v[16];
    reinterpret_cast<uint4*>(v)[0] = reinterpret_cast<const uint4*>(y + o)[0];
    reinterpret_cast<uint4*>(v)[1] = reinterpret_cast<const uint4*>(y + o)[1];
#pragma unroll
    for (int c = 0; c < 12; c++) tau[c * np + i] = s * (double)__bfloat162float(v[c]);
  }
}

// The closure's right-hand side in Fourier space (periodic box of side 2 pi, wave numbers m
// with the Nyquist index at +n/2 as the solver's): from the subgrid stress and electromotive
// force spectra (12 fields, laps_download_spectral layout),
//   momentum  f = -(i k . tau), projected on k-perpendicular (the incompressible solver's
//             pressure projection; 0 at k = 0)
//   induction g = i k x (eps + eps_Hall)
// into the 8 state fields (rho, rho u, B, p): 0, f, g, 0.
__global__ void k_closure_forcing(const double2* __restrict__ ts, double2* __restrict__ out, int n) {
  const int nh = n / 2 + 1;
  const long long ns = (long long)nh * n * n;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ns; i += (long long)gridDim.x * blockDim.x) {
    const int ix = (int)(i % nh), iy = (int)((i / nh) % n), iz = (int)(i / ((long long)nh * n));
    const double k[3] = {(double)ix, (double)(iy <= n / 2 ? iy : iy - n), (double)(iz <= n / 2 ? iz : iz - n)};
    double2 t[12];
#pragma unroll
    for (int c = 0; c < 12; c++) t[c] = ts[c * ns + i];
    // tau rows: (xx xy xz), (xy yy yz), (xz yz zz)
    const int idx[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
    double2 f[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
      double re = 0, im = 0;  // -i k_j tau_aj
#pragma unroll
      for (int j = 0; j < 3; j++) {
        re += k[j] * t[idx[a][j]].y;
        im -= k[j] * t[idx[a][j]].x;
      }
      f[a] = make_double2(re, im);
    }
    const double k2 = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
    if (k2 > 0.0) {
      const double dre = (k[0] * f[0].x + k[1] * f[1].x + k[2] * f[2].x) / k2;
      const double dim = (k[0] * f[0].y + k[1] * f[1].y + k[2] * f[2].y) / k2;
#pragma unroll
      for (int a = 0; a < 3; a++) f[a] = make_double2(f[a].x - k[a] * dre, f[a].y - k[a] * dim);
    } else {
      f[0] = f[1] = f[2] = make_double2(0.0, 0.0);
    }
    double2 e[3];
#pragma unroll
    for (int a = 0; a < 3; a++) e[a] = make_double2(t[6 + a].x + t[9 + a].x, t[6 + a].y + t[9 + a].y);
    // i (k x e): component a = i (k_b e_c - k_c e_b)
    double2 g[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
      const int b = (a + 1) % 3, c = (a + 2) % 3;
      const double cre = k[b] * e[c].x - k[c] * e[b].x, cim = k[b] * e[c].y - k[c] * e[b].y;
      g[a] = make_double2(-cim, cre);
    }
    out[i] = make_double2(0.0, 0.0);
#pragma unroll
    for (int a = 0; a < 3; a++) {
      out[(1 + a) * ns + i] = f[a];
      out[(4 + a) * ns + i] = g[a];
    }
    out[7 * ns + i] = make_double2(0.0, 0.0);
  }
}

// Packed weights of one layer, bf16 [tap][K chunk][N row][8], from fp32 w[co][ci][kz][ky][kx]
// (torch's Conv3d order; tap = (kz * 3 + ky) * 3 + kx; the layer computes the cross-correlation
// out[x] = sum w[k] in[x + k - 1]).  flip != 0 packs the weights of the input-gradient
// correlation: rows are input channels, columns output channels, taps mirrored.
__global__ void k_conv3_pack(const float* __restrict__ w, __nv_bfloat16* __restrict__ out, int cin, int cout, int kc, int np,
                             int flip) {
  const int tot = 27 * kc * np * 8;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < tot; i += gridDim.x * blockDim.x) {
    const int e = i % 8, n = (i / 8) % np, k = (i / (8 * np)) % kc, t = i / (8 * np * kc);
    const int ci_p = k * 8 + e;  // packed K index (channel of this layer's input)
    float v = 0.0f;
    if (!flip) {
      if (n < cout && ci_p < cin) v = w[((long long)n * cin + ci_p) * 27 + t];
    } else {  // input-gradient layer: its input channels are the forward outputs
      if (n < cin && ci_p < cout) v = w[((long long)ci_p * cin + n) * 27 + (26 - t)];
    }
    out[i] = __float2bfloat16_rn(v);
  }
}

// activations as a 2-D tensor {c channels, rows}: boxes of 8 channels (16 bytes) x box_rows rows
static CUtensorMap conv_tensor_map_box(const void* base, long long rows, int c, int box_rows) {
  CUtensorMap m;
  cuuint64_t dims[2] = {(cuuint64_t)c, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)c * 2};
  cuuint32_t box[2] = {8, (cuuint32_t)box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = tensor_map_encoder()(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, es,
                                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw Error{LAPS_ECUDA, "conv tensor map encoding failed (" + std::to_string((int)r) + ")"};
  return m;
}
static CUtensorMap conv_tensor_map(const void* base, long long rows, int c) {
  return conv_tensor_map_box(base, rows, c, CONV_TILE);
}

static __device__ int g_conv_err;

template <int KC, int NP>
static void launch_conv3(cudaStream_t s, const void* x, const void* wpk, ConvArgs a) {
  using CF = ConvCfg<KC, NP>;
  auto kern = k_conv3<KC, NP>;
  LAPS_CK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, CF::SMEM));
  LAPS_CK(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
  int per_sm = 0;
  LAPS_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, CONV_THREADS, CF::SMEM));
  int dev = 0, nsm = 0, smem_sm = 0;
  LAPS_CK(cudaGetDevice(&dev));
  LAPS_CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  LAPS_CK(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
  if (per_sm < 1) throw Error{LAPS_ECUDA, "conv kernel does not fit on an SM"};
  // the occupancy query answers for the default shared-memory carveout; with the full
  // carveout two blocks fit (128 registers x 192 threads, ~111 KB each): take the larger
  // count (blocks are independent, so blocks that do not fit at once only start later)
  if (per_sm < 2 && 2 * (CF::SMEM + 2048) <= smem_sm) per_sm = 2;
  const int grid = a.ntiles < nsm * per_sm ? a.ntiles : nsm * per_sm;
  const CUtensorMap tm = conv_tensor_map_box(x, (long long)a.nz * a.ny * (a.nx + 2), KC * 8, CF::A_ROWS);
  kern<<<grid, CONV_THREADS, CF::SMEM, s>>>(tm, reinterpret_cast<const uint4*>(wpk), a);
  LAPS_CK(cudaGetLastError());
}

template <int CI, int NP>
static void launch_wgrad(cudaStream_t s, const void* x, const void* dz, float* dw, int nx, int ny, int nz, int* err) {
  using CF = WgCfg<CI, NP>;
  auto kern = k_conv3_wgrad<CI, NP, LAPS_WGRAD_SWAP>;
  LAPS_CK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, CF::SMEM));
  LAPS_CK(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
  int dev = 0, nsm = 0;
  LAPS_CK(cudaGetDevice(&dev));
  LAPS_CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const int nchunks = nz * ny * (nx / WG_KV);
  int split = (2 * nsm + CF::GROUPS - 1) / CF::GROUPS;  // about two blocks per SM in all
  split = split < nchunks ? split : nchunks;
  const long long rows = (long long)nz * ny * (nx + 2);
  const CUtensorMap tx = conv_tensor_map_box(x, rows, CI, WG_KV);
  const CUtensorMap tz = conv_tensor_map_box(dz, rows, NP, WG_KV);
  LAPS_CK(cudaMemsetAsync(dw, 0, sizeof(float) * 27 * CI * NP, s));
  kern<<<dim3(CF::GROUPS, split), CONV_THREADS, CF::SMEM, s>>>(tx, tz, dw, nx, ny, nz, nchunks, err);
  LAPS_CK(cudaGetLastError());
}

}  // namespace laps

void laps_set_create_error(const std::string& m);

static bool conv_aligned(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

extern "C" int laps_conv3_pack(const float* w, void* wpk, int cin, int cout, int cin_p, int cout_p, int flip, void* stream) {
  using namespace laps;
  const int kin = flip ? cout_p : cin_p, nout = flip ? cin_p : cout_p;
  if (!w || !wpk || cin < 1 || cout < 1 || cin > cin_p || cout > cout_p || (cin_p != 16 && cin_p != 32) ||
      (cout_p != 16 && cout_p != 32) || !conv_aligned(wpk)) {
    laps_set_create_error("conv3 pack: null or unaligned buffer, or channels not within padded counts of 16 or 32");
    return LAPS_EINVAL;
  }
  try {
    k_conv3_pack<<<64, 256, 0, (cudaStream_t)stream>>>(w, reinterpret_cast<__nv_bfloat16*>(wpk), cin, cout, kin / 8, nout, flip);
    LAPS_CK(cudaGetLastError());
  } catch (const Error& e) {
    laps_set_create_error("conv3 pack: " + e.msg);
    return e.code;
  }
  return LAPS_OK;
}

extern "C" int laps_conv3_forward(const void* x, const void* wpk, const float* bias, void* y, void* zpre, const void* gate,
                                  int nx, int ny, int nz, int cin_p, int cout_p, int act, void* stream) {
  using namespace laps;
  if (!x || !wpk || !y || nx < CONV_TILE || nx % CONV_TILE || ny < 1 || nz < 1 || (cin_p != 16 && cin_p != 32) ||
      (cout_p != 16 && cout_p != 32) || act < 0 || act > 2 || (act == 2 && !gate) || !conv_aligned(x) ||
      !conv_aligned(wpk) || !conv_aligned(y) || (zpre && !conv_aligned(zpre)) || (gate && !conv_aligned(gate))) {
    laps_set_create_error("conv3 forward: bad argument (nx a multiple of 128; channels 16 or 32; act 0-2, act 2 needs a "
                          "gate; 16-byte aligned buffers)");
    return LAPS_EINVAL;
  }
  if ((long long)nz * ny * (nx + 2) >= (1LL << 31)) {
    laps_set_create_error("conv3 forward: grid too large");
    return LAPS_EINVAL;
  }
  try {
    void* ep = nullptr;
    LAPS_CK(cudaGetSymbolAddress(&ep, g_conv_err));
    ConvArgs a;
    a.nx = nx; a.ny = ny; a.nz = nz;
    a.ntiles = nz * ny * (nx / CONV_TILE);
    a.act = act;
    a.bias = bias;
    a.gate = reinterpret_cast<const __nv_bfloat16*>(gate);
    a.y = reinterpret_cast<__nv_bfloat16*>(y);
    a.zpre = reinterpret_cast<__nv_bfloat16*>(zpre);
    a.err = reinterpret_cast<int*>(ep);
    cudaStream_t s = (cudaStream_t)stream;
    if (cin_p == 16 && cout_p == 32) launch_conv3<2, 32>(s, x, wpk, a);
    else if (cin_p == 32 && cout_p == 32) launch_conv3<4, 32>(s, x, wpk, a);
    else if (cin_p == 32 && cout_p == 16) launch_conv3<4, 16>(s, x, wpk, a);
    else launch_conv3<2, 16>(s, x, wpk, a);
  } catch (const Error& e) {
    laps_set_create_error("conv3 forward: " + e.msg);
    return e.code;
  }
  return LAPS_OK;
}

extern "C" int laps_conv3_status(void* stream, int* err) {
  using namespace laps;
  try {
    LAPS_CK(cudaStreamSynchronize((cudaStream_t)stream));
    int h = 0, z = 0;
    LAPS_CK(cudaMemcpyFromSymbol(&h, g_conv_err, sizeof(int)));
    LAPS_CK(cudaMemcpyToSymbol(g_conv_err, &z, sizeof(int)));
    if (err) *err = h;
  } catch (const Error& e) {
    laps_set_create_error("conv3 status: " + e.msg);
    return e.code;
  }
  return LAPS_OK;
}

extern "C" int laps_conv3_wgrad(const void* x, const void* dz, float* dw, int nx, int ny, int nz, int cin_p, int cout_p,
                                void* stream) {
  using namespace laps;
  if (!x || !dz || !dw || nx < WG_KV || nx % WG_KV || ny < 1 || nz < 1 || (cin_p != 16 && cin_p != 32) ||
      (cout_p != 16 && cout_p != 32) || !conv_aligned(x) || !conv_aligned(dz) || !conv_aligned(dw)) {
    laps_set_create_error("conv3 wgrad: bad argument (nx a multiple of 64; channels 16 or 32; 16-byte aligned buffers)");
    return LAPS_EINVAL;
  }
  if ((long long)nz * ny * (nx + 2) >= (1LL << 31)) {
    laps_set_create_error("conv3 wgrad: grid too large");
    return LAPS_EINVAL;
  }
  try {
    void* ep = nullptr;
    LAPS_CK(cudaGetSymbolAddress(&ep, g_conv_err));
    cudaStream_t s = (cudaStream_t)stream;
    int* err = reinterpret_cast<int*>(ep);
    if (cin_p == 32 && cout_p == 32) launch_wgrad<32, 32>(s, x, dz, dw, nx, ny, nz, err);
    else if (cin_p == 32) launch_wgrad<32, 16>(s, x, dz, dw, nx, ny, nz, err);
    else if (cout_p == 32) launch_wgrad<16, 32>(s, x, dz, dw, nx, ny, nz, err);
    else launch_wgrad<16, 16>(s, x, dz, dw, nx, ny, nz, err);
  } catch (const Error& e) {
    laps_set_create_error("conv3 wgrad: " + e.msg);
    return e.code;
  }
  return LAPS_OK;
}

extern "C" int laps_closure_filter(const double* fine, int nfine, int ratio, double* coarse, float* targets, void* stream) {
  using namespace laps;
  if (!fine || !coarse || !targets || ratio < 1 || nfine < ratio || nfine % ratio) {
    laps_set_create_error("closure filter: null buffer or the fine size not a multiple of the ratio");
    return LAPS_EINVAL;
  }
  try {
    k_closure_filter<<<4 * 152, 256, 0, (cudaStream_t)stream>>>(fine, nfine, ratio, coarse, targets);
    LAPS_CK(cudaGetLastError());
  } catch (const Error& e) {
    laps_set_create_error("closure filter: " + e.msg);
    return e.code;
  }
  return LAPS_OK;
}

extern "C" int laps_closure_pack_input(const double* state, void* x, int n, double su, double sb, void* stream) {
  using namespace laps;
  if (!state || !x || n < 2 || !conv_aligned(x) || su <= 0 || sb <= 0) {
    laps_set_create_error("closure pack: bad argument");
    return LAPS_EINVAL;
  }
  try {
    k_closure_pack_input<<<4 * 152, 256, 0, (cudaStream_t)stream>>>(state, reinterpret_cast<__nv_bfloat16*>(x), n, su, sb);
    LAPS_CK(cudaGetLastError());
  } catch (const Error& e) {
    laps_set_create_error("closure pack: " + e.msg);
    return e.code;
  }
  return LAPS_OK;
}

extern "C" int laps_closure_unpack_output(const void* y, double* tau, int n, double s, void* stream) {
  using namespace laps;
  if (!y || !tau || n < 2 || !conv_aligned(y)) {
    laps_set_create_error("closure unpack: bad argument");
    return LAPS_EINVAL;
  }
  try {
    k_closure_unpack<<<4 * 152, 256, 0, (cudaStream_t)stream>>>(reinterpret_cast<const __nv_bfloat16*>(y), tau, n, s);
    LAPS_CK(cudaGetLastError());
  } catch (const Error& e) {
    laps_set_create_error("closure unpack: " + e.msg);
    return e.code;
  }
  return LAPS_OK;
}

extern "C" int laps_closure_forcing(const double* tau_spec, double* force_spec, int n, void* stream) {
  using namespace laps;
  if (!tau_spec || !force_spec || n < 2 || (n & (n - 1))) {
    laps_set_create_error("closure forcing: bad argument");
    return LAPS_EINVAL;
  }
  try {
    k_closure_forcing<<<4 * 152, 256, 0, (cudaStream_t)stream>>>(reinterpret_cast<const double2*>(tau_spec),
                                                                reinterpret_cast<double2*>(force_spec), n);
    LAPS_CK(cudaGetLastError());
  } catch (const Error& e) {
    laps_set_create_error("closure forcing: " + e.msg);
    return e.code;
  }
  return LAPS_OK;
}
