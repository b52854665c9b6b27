// Post-processing statistics of the state on the grid: the perpendicular angles between the
// increments of u and b = B / sqrt(<rho>) and between those of z+ = u - b and z- = u + b, as
// functions of the lag along one axis (theta_ub_zpm_perp_only,
// data_process/3D_C/statistics.c:10-356).  "Perpendicular" is with respect to the unit vector
// b0 = <B> / |<B>|.  For each lag l (1 <= l <= n_axis / 2) and each pair (a, b):
//   method 1: the mean of asin(|a_perp x b_perp| / (|a_perp| |b_perp|)) over the points where
//             both perpendicular parts are non-zero (:183-193);
//   method 2: asin(sum |a_perp x b_perp| / sum |a_perp| |b_perp|) over all points (:195-198,
//             :289-293).
// Float64 throughout.  Each block sums its points for one lag; a second kernel adds the block
// sums in a fixed order, so the result does not depend on scheduling.
#pragma once
#include <cstdint>

namespace laps {

constexpr int ANG_THREADS = 256;
constexpr int ANG_NSUM = 8;  // theta_ub, n_ub, num_ub, den_ub, theta_zpm, n_zpm, num_zpm, den_zpm

struct AngArgs {
  const double* u;  // ux, uy, uz fields (stride n)
  const double* B;  // Bx, By, Bz fields (stride n)
  long long n;
  int nx, ny, nz, axis, lag0;
  double sqrt_rho0;
  double b0x, b0y, b0z;
};

// perpendicular parts, their norms and the norm of their cross product (statistics.c:165-181)
__device__ __forceinline__ void ang_pair(const double a[3], const double b[3], double b0x, double b0y, double b0z,
                                         double& theta, double& cnt, double& num, double& den) {
  const double ad = a[0] * b0x + a[1] * b0y + a[2] * b0z;
  const double bd = b[0] * b0x + b[1] * b0y + b[2] * b0z;
  const double ap[3] = {a[0] - b0x * ad, a[1] - b0y * ad, a[2] - b0z * ad};
  const double bp[3] = {b[0] - b0x * bd, b[1] - b0y * bd, b[2] - b0z * bd};
  const double an = sqrt(ap[0] * ap[0] + ap[1] * ap[1] + ap[2] * ap[2]);
  const double bn = sqrt(bp[0] * bp[0] + bp[1] * bp[1] + bp[2] * bp[2]);
  const double c0 = ap[1] * bp[2] - ap[2] * bp[1];
  const double c1 = ap[2] * bp[0] - ap[0] * bp[2];
  const double c2 = ap[0] * bp[1] - ap[1] * bp[0];
  const double cn = sqrt(c0 * c0 + c1 * c1 + c2 * c2);
  if (an > 0 && bn > 0) {
    theta += asin(cn / (an * bn));
    cnt += 1.0;
  }
  num += cn;
  den += an * bn;
}

// grid (blocks, lags): block sums of lag lag0 + blockIdx.y into part[(lag, block)][8]
static __global__ void __launch_bounds__(ANG_THREADS) k_angle_partial(AngArgs a, double* __restrict__ part) {
  const int lag = a.lag0 + blockIdx.y;
  double s[ANG_NSUM] = {0, 0, 0, 0, 0, 0, 0, 0};
  const long long nxy = (long long)a.nx * a.ny;
  for (long long i = blockIdx.x * (long long)ANG_THREADS + threadIdx.x; i < a.n; i += (long long)gridDim.x * ANG_THREADS) {
    const int ix = (int)(i % a.nx), iy = (int)((i / a.nx) % a.ny), iz = (int)(i / nxy);
    long long j;
    if (a.axis == 0) j = i - ix + (ix + lag) % a.nx;
    else if (a.axis == 1) j = i + (long long)((iy + lag) % a.ny - iy) * a.nx;
    else j = i + (long long)((iz + lag) % a.nz - iz) * nxy;
    double du[3], db[3], zp[3], zm[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
      du[c] = a.u[c * a.n + j] - a.u[c * a.n + i];
      db[c] = (a.B[c * a.n + j] - a.B[c * a.n + i]) / a.sqrt_rho0;
      zp[c] = du[c] - db[c];
      zm[c] = du[c] + db[c];
    }
    ang_pair(du, db, a.b0x, a.b0y, a.b0z, s[0], s[1], s[2], s[3]);
    ang_pair(zp, zm, a.b0x, a.b0y, a.b0z, s[4], s[5], s[6], s[7]);
  }
  __shared__ double red[ANG_THREADS / 32][ANG_NSUM];
#pragma unroll
  for (int k = 0; k < ANG_NSUM; k++) {
    double v = s[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < ANG_NSUM) {
    double v = 0;
    for (int w = 0; w < ANG_THREADS / 32; w++) v += red[w][threadIdx.x];
    part[((long long)blockIdx.y * gridDim.x + blockIdx.x) * ANG_NSUM + threadIdx.x] = v;
  }
}

// one thread per lag: the block sums in block order, then the two methods (statistics.c:338-349)
static __global__ void k_angle_final(const double* __restrict__ part, int nblk, int nlag, int lag0, int naxis, double* __restrict__ out) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nlag) return;
  double s[ANG_NSUM] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int b = 0; b < nblk; b++)
#pragma unroll
    for (int k = 0; k < ANG_NSUM; k++) s[k] += part[((long long)q * nblk + b) * ANG_NSUM + k];
  const int l = lag0 + q;
  out[0 * naxis + l] = s[0] / s[1];
  out[1 * naxis + l] = asin(s[2] / s[3]);
  out[2 * naxis + l] = s[4] / s[5];
  out[3 * naxis + l] = asin(s[6] / s[7]);
}

// <rho>, <Bx>, <By>, <Bz>: the k = 0 coefficients of the state (the forward transform is
// normalised by the number of grid points)
template <class TS>
__global__ void k_state_means(const typename Store<TS>::C* __restrict__ U, long long fsc, double* __restrict__ out) {
  const int f[4] = {0, 4, 5, 6};
  if (threadIdx.x < 4) out[threadIdx.x] = Real<TS>::to_d(Store<TS>::ldc(U + f[threadIdx.x] * fsc).re);
}

}  // namespace laps
