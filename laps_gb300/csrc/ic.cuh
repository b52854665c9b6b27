// Fresh-start initial conditions on the device: the reference's background fields
// (background_fields_initialize, src_compressible/mhdinit.f90:183-299) and perturbations
// (perturbation_initialize, :302-1036, cases 1, 6, 7, 8), then the primitive -> conserved
// conversion (:1038-1056).  The random-phase mode sums of cases 6 and 7 arrive as real fields
// (rho, u, B perturbations) that the host placed in the half spectrum and the state's inverse
// transform brought to the grid; everything pointwise happens here, in float64.
#pragma once
#include "engine.cuh"

namespace laps {

struct IcDev {
  laps_ic ic;
  double Lx, Ly, Lz;
  double cosc, sinc;  // corotation angle (AEBmod.f90:28-33)
  double gamma;
  int incomp;         // 3-D incompressible: ipert 1 in its own form, p kept in slot 8
  int modes;          // the 7 perturbation fields of ipert 6 / 7 are in the input
};

// primitive background at grid point (x, y, z): mhdinit.f90:199-296
__device__ inline void ic_background(const IcDev& d, double x, double y, double z, double v[8]) {
  const laps_ic& c = d.ic;
  const double ninf = 1.0;
  for (int f = 0; f < 8; f++) v[f] = 0.0;
  v[0] = c.rho0;
  v[7] = c.rho0 * c.T0;
  switch (c.ifield) {
    case 1: {  // double current sheet Bx(z), density carries the pressure balance
      const double zc = 0.5 * d.Lz, zz = z < zc ? z - 0.25 * d.Lz : z - 0.75 * d.Lz, sg = z < zc ? 1.0 : -1.0;
      v[4] = sg * c.B0 * tanh(zz / c.a0);
      const double ch = cosh(zz / c.a0);
      v[0] = ninf + c.B0 * c.B0 / 2.0 / c.T0 / (ch * ch);
      v[7] = v[0] * c.T0;
      break;
    }
    case 2: {  // double Harris shear ux(y), rho(y); a0 = Ly shear_width / 2
      const double a = d.Ly * 0.5 * c.shear_width;
      const double yc = 0.5 * d.Ly, yy = y < yc ? y - 0.25 * d.Ly : y - 0.75 * d.Ly, sg = y < yc ? 1.0 : -1.0;
      const double t = tanh(yy / a);
      v[1] = sg * 0.5 * (c.U_fast - c.U_slow) * t + 0.5 * (c.U_fast + c.U_slow);
      v[0] = sg * 0.5 * (c.n_fast - c.n_slow) * t + 0.5 * (c.n_fast + c.n_slow);
      v[7] = c.press0;
      v[4] = c.bx0;
      v[5] = c.by0;
      break;
    }
    case 3:  // uniform B
      v[4] = c.bx0; v[5] = c.by0; v[6] = c.bz0; v[7] = c.press0;
      break;
    case 4: {  // double current sheet Bx(y), uniform density
      const double yc = 0.5 * d.Ly, yy = y < yc ? y - 0.25 * d.Ly : y - 0.75 * d.Ly, sg = y < yc ? 1.0 : -1.0;
      v[4] = sg * c.B0 * tanh(yy / c.a0);
      v[7] = c.press0 - 0.5 * v[4] * v[4];
      v[0] = ninf;
      break;
    }
    case 5: {  // jet along x (3-D compressible only)
      v[4] = c.bx0; v[5] = c.by0; v[6] = c.bz0; v[7] = c.press0;
      const double dz = z - d.Lz / 2, dy = y - d.Ly / 2;
      const double r = sqrt(dz * dz + dy * dy);
      v[1] = c.Vjet / 2 * (1 - tanh((r - 1) / 0.1));
      break;
    }
    default:
      break;
  }
}

// ipert 1, circularly polarised Alfven wave: mhdinit.f90:328-342
// (src_incompressible/mhdinit.f90:318-333: B scaled by sqrt(rho), u not, wave number 1)
__device__ inline void ic_alfven(const IcDev& d, double x, double v[8]) {
  const laps_ic& c = d.ic;
  const double pi = 3.141592653589793;
  const double kx = d.incomp ? 2 * pi / d.Lx : 2 * pi / d.Lx * c.wave_number_jet;
  const double s = sin(kx * x), co = cos(kx * x), sr = sqrt(v[0]);
  if (d.incomp) {
    v[6] = v[6] - c.db0 * sr * s;
    v[3] = v[3] + c.db0 * s;
    v[1] = v[1] + c.db0 * co * d.sinc;
    v[4] = v[4] - c.db0 * sr * co * d.sinc;
    v[2] = v[2] + c.db0 * co * d.cosc;
    v[5] = v[5] - c.db0 * sr * co * d.cosc;
  } else {
    v[6] = v[6] - c.db0 * s;
    v[3] = v[3] + c.db0 / sr * s;
    v[1] = v[1] + c.db0 / sr * co * d.sinc;
    v[4] = v[4] - c.db0 * co * d.sinc;
    v[2] = v[2] + c.db0 / sr * co * d.cosc;
    v[5] = v[5] - c.db0 * co * d.cosc;
  }
}

// ipert 8, a switchback along x over a flux-tube profile in r = |(y, z) - centre|, with the
// velocity anti-correlated to B: mhdinit.f90:931-1019.  Components are rotated as the
// reference notes (its Bz_SB is added to Bx, Bx_SB to By, By_SB to Bz).
__device__ inline void ic_switchback(const IcDev& d, double x, double y, double z, double v[8]) {
  const laps_ic& c = d.ic;
  const double pi = 3.141592653589793, spi = sqrt(pi);
  const double zs = z - d.Lz / 2, ys = y - d.Ly / 2, xs = x - d.Lx / 2;
  const double r = sqrt(ys * ys + zs * zs);
  const double e0 = (r - c.R0_SB) / c.R1_SB, ex = xs / c.H_SB;
  const double Bz0 = c.B0_SB + c.dB_SB * exp(-e0 * e0);
  double Bz = c.B0_SB + c.dB_SB * exp(-e0 * e0 - ex * ex);
  const double Cs = -(exp(-(c.R0_SB / c.R1_SB) * (c.R0_SB / c.R1_SB)) + spi * c.R0_SB / c.R1_SB * erf(c.R0_SB / c.R1_SB));
  double phi = 0.0, Br = 0.0, Bphi = 0.0;
  if (!(r < 1e-8)) {
    phi = atan2(zs, ys);
    const double G = exp(-e0 * e0) + spi * c.R0_SB / c.R1_SB * erf((c.R0_SB - r) / c.R1_SB) + Cs;
    Br = -c.dB_SB * (xs * c.R1_SB * c.R1_SB) / (r * c.H_SB * c.H_SB) * exp(-ex * ex) * G;
    double p, q;
    if (r < c.Rm_SB) {
      p = 1;
      q = 1;
    } else {
      const double er = (r - c.Rm_SB) / c.Rd_SB;
      p = exp(-er * er);
      const double dpdr = -2 * (r - c.Rm_SB) / (c.Rd_SB * c.Rd_SB) * p;
      q = Bz0 / Bz * (1 + 1 / Bz0 * (p * (Bz - Bz0) - (dpdr * c.dB_SB * c.R1_SB * c.R1_SB / r * G * 0.5 * (exp(-ex * ex) - 1))));
    }
    Br = Br * p;
    Bz = Bz * q;
    if (Bz * Bz + Br * Br < c.B0_SB * c.B0_SB) {
      Bphi = sqrt(c.B0_SB * c.B0_SB - Br * Br - Bz * Bz);
    } else {
      Bphi = 0.0;
      v[7] = v[7] - 0.5 * (Bz * Bz + Br * Br - c.B0_SB * c.B0_SB);  // keeps the total pressure
    }
  }
  const double Bx = Br * cos(phi) - Bphi * sin(phi);
  const double By = Br * sin(phi) + Bphi * cos(phi);
  v[4] += Bz;
  v[5] += Bx;
  v[6] += By;
  const double sr = sqrt(v[0]);
  v[1] -= v[4] / sr;
  v[2] -= v[5] / sr;
  v[3] -= v[6] / sr;
}

// one thread per grid point: w holds the 7 mode-sum fields (rho, u, B) when d.modes, and
// receives the 8 conserved fields (storage type TS) in place
template <class TS>
__global__ void k_init_fields(typename Store<TS>::R* __restrict__ w, Geo g, IcDev d) {
  const long long n = g.fsr;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int ix = (int)(i % g.nx), iy = (int)((i / g.nx) % g.ny), iz = (int)(i / ((long long)g.nx * g.ny));
    const double x = ix * (d.Lx / g.nx), y = iy * (d.Ly / g.ny), z = iz * (d.Lz / g.nz);
    double v[8];
    ic_background(d, x, y, z, v);
    if (d.ic.ipert == 1) ic_alfven(d, x, v);
    else if (d.ic.ipert == 8) ic_switchback(d, x, y, z, v);
    if (d.modes) {
#pragma unroll
      for (int f = 0; f < 7; f++) v[f] += Real<TS>::to_d(Store<TS>::ld(w + f * n + i));
    }
    // initial_calc_conserve_variable (the incompressible state keeps p in slot 8)
    const double ux = v[1], uy = v[2], uz = v[3], p = v[7];
    v[1] = v[0] * ux;
    v[2] = v[0] * uy;
    v[3] = v[0] * uz;
    if (!d.incomp) v[7] = p / (d.gamma - 1) + 0.5 * (v[0] * (ux * ux + uy * uy + uz * uz) + v[4] * v[4] + v[5] * v[5] + v[6] * v[6]);
#pragma unroll
    for (int f = 0; f < 8; f++) Store<TS>::st(w + f * n + i, Real<TS>::from_d(v[f]));
  }
}

// the host-placed half-spectrum coefficients of the mode sums: entry e adds val[e * 7 + f]
// (float64 complex) to field f at spectral offset idx[e] (z, y, kx) of the state buffer
template <class TS>
__global__ void k_place_modes(typename Store<TS>::C* __restrict__ u, long long fsc, const long long* __restrict__ idx,
                              const double2* __restrict__ val, int count) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < count; e += gridDim.x * blockDim.x) {
#pragma unroll
    for (int f = 0; f < 7; f++) {
      const double2 c = val[(long long)e * 7 + f];
      Store<TS>::stc(u + f * fsc + idx[e], cx<TS>{Real<TS>::from_d(c.x), Real<TS>::from_d(c.y)});
    }
  }
}

}  // namespace laps
