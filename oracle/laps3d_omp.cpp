// CPU restatement (oracle O2) of LAPS's 3-D compressible RHS evaluation and RK3 time advance,
// in C++ with OpenMP threads and its own FFT.
//
// TEST AND BASELINE INFRASTRUCTURE ONLY.  Nothing in the shipped GPU path links or calls
// this file; the benchmark times it as the CPU baseline ("port": a restatement, not the
// reference binary, which needs Fortran, MPI and FFTW that neither machine has), and the
// CPU tests check it against the numpy restatement (oracle/laps3d.py).  Parity unpinned,
// as for that restatement: the reference ships no golden vectors.
//
// It follows the reference's routines (file:line inside the reference project) in FP64:
//   transform_uu_real_to_fourier / _fourier_to_real   src_compressible/fftw.f90:42-103
//   calc_flux (+ expansion term, Hall E)              src_compressible/mhdrhs.f90:21-124
//   calc_current_density_real                         src_compressible/mhdrhs.f90:296-362
//   transform_flux_real_to_fourier                    src_compressible/mhdrhs.f90:128-172
//   calc_rhs                                          src_compressible/mhdrhs.f90:174-279
//   update_uu_prim_from_uu                            src_compressible/mhdrhs.f90:282-294
//   rkt_init / rkt                                    src_compressible/rktmod.f90:15-62
//   dealias (option 1, the 2/3 sphere)                src_compressible/dealiasing.f90:13-113
//   evolve_radius / update_ksquare (no corotation)    src_compressible/AEBmod.f90:46-125
//   vardt                                             src_compressible/mhd.f90:328-429
//   evolve                                            src_compressible/mhd.f90:298-326
// Scope: the options the 3-D compressible benchmark case uses - implicit viscosity and
// resistivity, dealias option 1, Hall term, expanding box without corotation.  Other options
// are rejected at creation.
//
// FFTs: complex radix-2 decimation-in-time transforms with twiddles from long-double sin/cos;
// two real x rows are transformed as one complex line (z = a + i b) and separated, and the
// inverse builds the pair's Hermitian line from the two half spectra, ignoring the imaginary
// parts of the DC and Nyquist inputs as FFTW's c2r does.  Forward normalisation per axis
// (fftw.f90:62,160,177).  Columns are gathered 16 at a time into contiguous buffers.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>
#include <omp.h>

namespace {

using cd = std::complex<double>;
const double PI = 3.141592653589793;  // mhdinit.f90:7

struct Fft {
  int n = 0, logn = 0;
  std::vector<cd> tw;   // exp(-2 pi i j / n), j < n/2
  std::vector<int> rev;
  void init(int n_) {
    n = n_;
    logn = 0;
    while ((1 << logn) < n) logn++;
    tw.resize(n / 2 > 0 ? n / 2 : 1);
    for (int j = 0; j < n / 2; j++) {
      long double a = 2.0L * 3.141592653589793238462643383279502884L * j / n;
      tw[j] = cd((double)cosl(a), (double)-sinl(a));
    }
    rev.resize(n);
    for (int i = 0; i < n; i++) {
      int r = 0;
      for (int b = 0; b < logn; b++) r |= ((i >> b) & 1) << (logn - 1 - b);
      rev[i] = r;
    }
  }
  // in place, unnormalised: sign -1 forward (exp(-i)), +1 backward
  void run(cd* a, int sign) const {
    for (int i = 0; i < n; i++)
      if (i < rev[i]) std::swap(a[i], a[rev[i]]);
    for (int len = 2; len <= n; len <<= 1) {
      const int half = len >> 1, step = n / len;
      for (int i = 0; i < n; i += len) {
        for (int j = 0; j < half; j++) {
          cd w = tw[j * step];
          if (sign > 0) w = std::conj(w);
          const cd u = a[i + j], v = a[i + j + half] * w;
          a[i + j] = u + v;
          a[i + j + half] = u - v;
        }
      }
    }
  }
};

struct Params {
  int nx, ny, nz;
  double gamma, eta, nu, cfl, R0, Ur0, di;
  int if_resis, if_visc, if_AEB, if_Hall;
};

struct Solver {
  Params p;
  int nh;
  long long nr, ns;  // real points, spectral points per field
  double dx, dy, dz;
  std::vector<double> wx, wy, wz;
  std::vector<unsigned char> keep;
  Fft fx, fy, fz;
  std::vector<double> uu, prim, flux, jr;  // 8, 4, 19, 3 real fields
  std::vector<cd> uf, ff, fnl, fnl_rk, jf;  // 8, 19, 8, 8, 3 spectral fields
  std::vector<double> ksq;
  double cc1[3], dd1[3], ts[3];
  double dt = 0.0, time = 0.0, radius = 0.0, tau = 0.0;

  double* U(int f) { return uu.data() + f * nr; }
  cd* UF(int f) { return uf.data() + f * ns; }

  static std::vector<double> wave_numbers(int n, double L) {  // mhdinit.f90:88-115 (Nyquist +k)
    std::vector<double> w(n);
    for (int i = 0; i < n; i++) w[i] = i <= n / 2 ? (2 * PI * i) / L : (2 * PI * (i - n)) / L;
    return w;
  }

  explicit Solver(const Params& q) : p(q) {
    nh = p.nx / 2 + 1;
    nr = (long long)p.nx * p.ny * p.nz;
    ns = (long long)nh * p.ny * p.nz;
    const double L = 2 * PI;
    dx = L / p.nx; dy = L / p.ny; dz = L / p.nz;
    wx = wave_numbers(p.nx, L); wx.resize(nh);
    wy = wave_numbers(p.ny, L);
    wz = wave_numbers(p.nz, L);
    fx.init(p.nx); fy.init(p.ny); fz.init(p.nz);
    keep.resize(ns);
    for (int k = 0; k < p.nz; k++)
      for (int j = 0; j < p.ny; j++)
        for (int i = 0; i < nh; i++) {  // dealiasing.f90:87-99 (option 1)
          double rx = wx[i] * L / (2 * PI * p.nx), ry = wy[j] * L / (2 * PI * p.ny), rz = wz[k] * L / (2 * PI * p.nz);
          double rad = std::sqrt((rx * rx + ry * ry) + rz * rz);
          keep[((long long)k * p.ny + j) * nh + i] = !(rad > 1.0 / 3.0);
        }
    uu.assign(8 * nr, 0.0); prim.assign(4 * nr, 0.0); flux.assign(19 * nr, 0.0); jr.assign(3 * nr, 0.0);
    uf.assign(8 * ns, 0.0); ff.assign(19 * ns, 0.0); fnl.assign(8 * ns, 0.0); fnl_rk.assign(8 * ns, 0.0);
    jf.assign(3 * ns, 0.0);
    ksq.assign(ns, 0.0);
    radius = p.R0;
    tau = p.Ur0 != 0.0 ? radius / p.Ur0 : INFINITY;
    evolve_radius(0.0);
  }

  // AEBmod.f90:56-73,87-125 (no corotation)
  void evolve_radius(double t) {
    const double Ur = p.if_AEB ? p.Ur0 : 0.0;
    radius = p.R0 + Ur * t;
    tau = Ur != 0.0 ? radius / Ur : INFINITY;
    const double rr = p.R0 / radius;
#pragma omp parallel for
    for (int k = 0; k < p.nz; k++)
      for (int j = 0; j < p.ny; j++)
        for (int i = 0; i < nh; i++) {
          const double kx = wx[i], ky = wy[j] * rr, kz = wz[k] * rr;
          ksq[((long long)k * p.ny + j) * nh + i] = kx * kx + ky * ky + kz * kz;
        }
  }

  // ------------------------------------------------------------------ transforms
  // real (nz, ny, nx) -> half spectrum (nz, ny, nh), each axis divided by its length
  void forward(const double* in, cd* out) {
    const int nx = p.nx, ny = p.ny, nz = p.nz;
    const long long rows = (long long)ny * nz;
#pragma omp parallel
    {
      std::vector<cd> z(nx);
#pragma omp for
      for (long long r = 0; r < rows; r += 2) {  // two real rows per complex line
        const double* a = in + r * nx;
        const double* b = in + (r + 1) * nx;
        for (int j = 0; j < nx; j++) z[j] = cd(a[j], b[j]);
        fx.run(z.data(), -1);
        cd* oa = out + r * nh;
        cd* ob = out + (r + 1) * nh;
        for (int k = 0; k < nh; k++) {
          const cd zk = z[k], zm = std::conj(z[(nx - k) % nx]);
          oa[k] = 0.5 * (zk + zm) / (double)nx;
          ob[k] = cd(0.0, -0.5) * (zk - zm) / (double)nx;
        }
      }
    }
    columns(out, -1, true);
  }
  // half spectrum -> real, unnormalised: z, y c2c, x c2r (fftw.f90:182-222,94-99); `in` is
  // overwritten by the column passes
  void inverse(cd* in, double* out) {
    const int nx = p.nx, ny = p.ny, nz = p.nz;
    columns(in, +1, false);
    const long long rows = (long long)ny * nz;
#pragma omp parallel
    {
      std::vector<cd> z(nx);
#pragma omp for
      for (long long r = 0; r < rows; r += 2) {
        const cd* A = in + r * nh;
        const cd* B = in + (r + 1) * nh;
        for (int k = 0; k < nh; k++) {
          cd a = A[k], b = B[k];
          if (k == 0 || k == nx / 2) { a = cd(a.real(), 0.0); b = cd(b.real(), 0.0); }
          z[k] = a + cd(0.0, 1.0) * b;
          if (k > 0 && k < nx / 2) z[nx - k] = std::conj(a) + cd(0.0, 1.0) * std::conj(b);
        }
        fx.run(z.data(), +1);
        double* oa = out + r * nx;
        double* ob = out + (r + 1) * nx;
        for (int j = 0; j < nx; j++) { oa[j] = z[j].real(); ob[j] = z[j].imag(); }
      }
    }
  }
  // y and z c2c of a half spectrum in place; forward: y then z, each divided by its length;
  // backward: z then y, unnormalised
  void columns(cd* w, int sign, bool fwd) {
    const int ny = p.ny, nz = p.nz;
    constexpr int CB = 16;
    auto ypass = [&]() {
#pragma omp parallel
      {
        std::vector<cd> buf((size_t)CB * ny), line(ny);
#pragma omp for collapse(2)
        for (int k = 0; k < nz; k++)
          for (int i0 = 0; i0 < nh; i0 += CB) {
            const int nb = std::min(CB, nh - i0);
            cd* plane = w + (long long)k * ny * nh;
            for (int j = 0; j < ny; j++)
              for (int c = 0; c < nb; c++) buf[(size_t)c * ny + j] = plane[(long long)j * nh + i0 + c];
            for (int c = 0; c < nb; c++) {
              fy.run(buf.data() + (size_t)c * ny, sign);
              if (fwd)
                for (int j = 0; j < ny; j++) buf[(size_t)c * ny + j] /= (double)ny;
            }
            for (int j = 0; j < ny; j++)
              for (int c = 0; c < nb; c++) plane[(long long)j * nh + i0 + c] = buf[(size_t)c * ny + j];
          }
      }
    };
    auto zpass = [&]() {
      const long long zs = (long long)ny * nh;
#pragma omp parallel
      {
        std::vector<cd> buf((size_t)CB * nz);
#pragma omp for collapse(2)
        for (int j = 0; j < ny; j++)
          for (int i0 = 0; i0 < nh; i0 += CB) {
            const int nb = std::min(CB, nh - i0);
            cd* col = w + (long long)j * nh + i0;
            for (int k = 0; k < nz; k++)
              for (int c = 0; c < nb; c++) buf[(size_t)c * nz + k] = col[k * zs + c];
            for (int c = 0; c < nb; c++) {
              fz.run(buf.data() + (size_t)c * nz, sign);
              if (fwd)
                for (int k = 0; k < nz; k++) buf[(size_t)c * nz + k] /= (double)nz;
            }
            for (int k = 0; k < nz; k++)
              for (int c = 0; c < nb; c++) col[k * zs + c] = buf[(size_t)c * nz + k];
          }
      }
    };
    if (fwd) { ypass(); zpass(); } else { zpass(); ypass(); }
  }

  // ------------------------------------------------------------------ state
  void set_primitive(const double* pr) {  // mhdinit.f90:1038-1056
    const double g = p.gamma;
    std::memcpy(uu.data(), pr, sizeof(double) * 8 * nr);
#pragma omp parallel for
    for (long long i = 0; i < nr; i++) {
      const double rho = pr[i], ux = pr[nr + i], uy = pr[2 * nr + i], uz = pr[3 * nr + i];
      const double bx = pr[4 * nr + i], by = pr[5 * nr + i], bz = pr[6 * nr + i], P = pr[7 * nr + i];
      prim[i] = ux; prim[nr + i] = uy; prim[2 * nr + i] = uz; prim[3 * nr + i] = P;
      uu[nr + i] = rho * ux; uu[2 * nr + i] = rho * uy; uu[3 * nr + i] = rho * uz;
      uu[7 * nr + i] = P / (g - 1) + 0.5 * (rho * (ux * ux + uy * uy + uz * uz) + bx * bx + by * by + bz * bz);
    }
    for (int f = 0; f < 8; f++) forward(U(f), UF(f));
  }
  void update_prim() {  // mhdrhs.f90:282-294
    const double g = p.gamma;
#pragma omp parallel for
    for (long long i = 0; i < nr; i++) {
      const double rho = uu[i];
      const double ux = uu[nr + i] / rho, uy = uu[2 * nr + i] / rho, uz = uu[3 * nr + i] / rho;
      const double bx = uu[4 * nr + i], by = uu[5 * nr + i], bz = uu[6 * nr + i];
      prim[i] = ux; prim[nr + i] = uy; prim[2 * nr + i] = uz;
      prim[3 * nr + i] = (uu[7 * nr + i] - 0.5 * (uu[nr + i] * ux + uu[2 * nr + i] * uy + uu[3 * nr + i] * uz +
                                                  bx * bx + by * by + bz * bz)) * (g - 1);
    }
  }
  void to_real() {  // transform_uu_fourier_to_real on a copy (the inverse overwrites its input)
    for (int f = 0; f < 8; f++) {
      std::memcpy(fnl.data(), UF(f), sizeof(cd) * ns);
      inverse(fnl.data(), U(f));
    }
  }

  // ------------------------------------------------------------------ mhdrhs.f90
  void calc_flux() {
    const double g = p.gamma;
    if (p.if_Hall) {  // J = ik x B (mhdrhs.f90:296-362), ky and kz scaled by R0/R
      const double rr = p.R0 / radius;
#pragma omp parallel for
      for (int k = 0; k < p.nz; k++)
        for (int j = 0; j < p.ny; j++)
          for (int i = 0; i < nh; i++) {
            const long long s = ((long long)k * p.ny + j) * nh + i;
            const cd I(0.0, 1.0);
            const double kx = wx[i], ky = wy[j] * rr, kz = wz[k] * rr;
            const cd bx = UF(4)[s], by = UF(5)[s], bz = UF(6)[s];
            jf[s] = I * ky * bz - I * kz * by;
            jf[ns + s] = I * kz * bx - I * kx * bz;
            jf[2 * ns + s] = I * kx * by - I * ky * bx;
          }
      for (int c = 0; c < 3; c++) inverse(jf.data() + c * ns, jr.data() + c * nr);
    }
    const double di = p.di;
#pragma omp parallel for
    for (long long i = 0; i < nr; i++) {
      const double rho = uu[i], mx = uu[nr + i], my = uu[2 * nr + i], mz = uu[3 * nr + i];
      const double Bx = uu[4 * nr + i], By = uu[5 * nr + i], Bz = uu[6 * nr + i], e = uu[7 * nr + i];
      const double ux = prim[i], uy = prim[nr + i], uz = prim[2 * nr + i], P = prim[3 * nr + i];
      const double ptot = P + 0.5 * (Bx * Bx + By * By + Bz * Bz);
      const double udotb = ux * Bx + uy * By + uz * Bz;
      double* f = flux.data();
      f[i] = mx; f[nr + i] = my; f[2 * nr + i] = mz;
      f[3 * nr + i] = mx * ux - Bx * Bx + ptot;
      f[4 * nr + i] = my * ux - By * Bx;
      f[5 * nr + i] = mz * ux - Bz * Bx;
      f[6 * nr + i] = mx * uy - Bx * By;
      f[7 * nr + i] = my * uy - By * By + ptot;
      f[8 * nr + i] = mz * uy - Bz * By;
      f[9 * nr + i] = mx * uz - Bx * Bz;
      f[10 * nr + i] = my * uz - By * Bz;
      f[11 * nr + i] = mz * uz - Bz * Bz + ptot;
      double ex = uz * By - uy * Bz, ey = ux * Bz - uz * Bx, ez = uy * Bx - ux * By;
      if (p.if_Hall) {
        const double jx = jr[i], jy = jr[nr + i], jz = jr[2 * nr + i];
        ex = ex + di / rho * (jy * Bz - jz * By);
        ey = ey + di / rho * (jz * Bx - jx * Bz);
        ez = ez + di / rho * (jx * By - jy * Bx);
      }
      f[12 * nr + i] = ex; f[13 * nr + i] = ey; f[14 * nr + i] = ez;
      f[15 * nr + i] = (e + ptot) * ux - udotb * Bx;
      f[16 * nr + i] = (e + ptot) * uy - udotb * By;
      f[17 * nr + i] = (e + ptot) * uz - udotb * Bz;
      if (p.if_AEB)  // mhdrhs.f90:93-103
        f[18 * nr + i] = -2 * g / (g - 1) * P / tau - (2.0 * Bx * Bx + By * By + Bz * Bz) / tau -
                         (mx * ux + 2 * my * uy + 2 * mz * uz) / tau;
    }
    const int nf = p.if_AEB ? 19 : 18;
    for (int f = 0; f < nf; f++) forward(flux.data() + f * nr, ff.data() + f * ns);
  }

  void calc_rhs() {  // mhdrhs.f90:174-279 (no explicit diffusion)
    const double rr = p.R0 / radius;
    static const double ebm[7] = {2.0, 2.0, 3.0, 3.0, 2.0, 1.0, 1.0};
#pragma omp parallel for
    for (int k = 0; k < p.nz; k++)
      for (int j = 0; j < p.ny; j++)
        for (int i = 0; i < nh; i++) {
          const long long s = ((long long)k * p.ny + j) * nh + i;
          const cd I(0.0, 1.0);
          const cd ikx = I * wx[i], iky = I * (wy[j] * rr), ikz = I * (wz[k] * rr);
          auto F = [&](int f) { return ff[f * ns + s]; };
          cd r[8];
          r[0] = -(ikx * F(0) + iky * F(1) + ikz * F(2));
          r[1] = -(ikx * F(3) + iky * F(4) + ikz * F(5));
          r[2] = -(ikx * F(6) + iky * F(7) + ikz * F(8));
          r[3] = -(ikx * F(9) + iky * F(10) + ikz * F(11));
          r[4] = ikz * F(13) - iky * F(14);
          r[5] = ikx * F(14) - ikz * F(12);
          r[6] = iky * F(12) - ikx * F(13);
          r[7] = -(ikx * F(15) + iky * F(16) + ikz * F(17));
          if (p.if_AEB) {
            for (int v = 0; v < 7; v++) r[v] = r[v] - ebm[v] * UF(v)[s] / tau;
            r[7] = r[7] + F(18);
          }
          for (int v = 0; v < 8; v++) fnl[v * ns + s] = r[v];
        }
  }

  // ------------------------------------------------------------------ rktmod.f90, dealias
  void rkt_init() {
    std::fill(fnl_rk.begin(), fnl_rk.end(), cd(0.0, 0.0));
    cc1[0] = 8.0 / 15.0 * dt; cc1[1] = 5.0 / 12.0 * dt; cc1[2] = 0.75 * dt;
    dd1[0] = 0.0; dd1[1] = -17.0 / 60.0 * dt; dd1[2] = -5.0 / 12.0 * dt;
    ts[0] = 8.0 / 15.0 * dt; ts[1] = 2.0 / 15.0 * dt; ts[2] = 1.0 / 3.0 * dt;
  }
  void rkt_dealias(int k) {
#pragma omp parallel for
    for (long long s = 0; s < ns; s++) {
      for (int v = 0; v < 8; v++) {
        cd u = cc1[k] * fnl[v * ns + s] + dd1[k] * fnl_rk[v * ns + s] + UF(v)[s];
        fnl_rk[v * ns + s] = fnl[v * ns + s];
        if (v >= 1 && v <= 3 && p.if_visc) u = u / (ts[k] * ksq[s] * p.nu + 1.0);
        if (v >= 4 && v <= 6 && p.if_resis) u = u / (ts[k] * ksq[s] * p.eta + 1.0);
        if (!keep[s]) u = 0.0;
        UF(v)[s] = u;
      }
    }
  }

  // ------------------------------------------------------------------ mhd.f90
  double vardt_min() {  // mhd.f90:350-419
    const double g = p.gamma, s2 = std::sqrt(2.0);
    const double mind = std::min(dx, std::min(dy, dz));
    const double fy = radius / p.R0;
    double best = INFINITY;
#pragma omp parallel for reduction(min : best)
    for (long long i = 0; i < nr; i++) {
      const double rho = uu[i];
      const double cs2 = g * prim[3 * nr + i] / rho, sq = std::sqrt(rho);
      const double ca[3] = {uu[4 * nr + i] / sq, uu[5 * nr + i] / sq, uu[6 * nr + i] / sq};
      const double ca2 = ca[0] * ca[0] + ca[1] * ca[1] + ca[2] * ca[2];
      const double cms2 = cs2 + ca2;
      // Hall speed with the signed max of B (mhd.f90:392-399)
      const double ch = p.if_Hall ? p.di / rho * std::max(std::max(uu[4 * nr + i], uu[5 * nr + i]), uu[6 * nr + i]) / mind : 0.0;
      for (int a = 0; a < 3; a++) {
        const double u = prim[a * nr + i];
        const double cns2 = std::sqrt(std::max(cms2 * cms2 - 4 * cs2 * ca[a] * ca[a], 0.0));
        const double cf = std::sqrt(cms2 + cns2) / s2, csl = std::sqrt(std::max(cms2 - cns2, 0.0)) / s2;
        double c = std::max({std::abs(u + cf), std::abs(u + csl), std::abs(u + ca[a]), std::abs(u - cf),
                             std::abs(u - csl), std::abs(u - ca[a]), std::abs(u)});
        if (p.if_Hall) c = std::max(c, ch);
        const double t = (a == 0 ? dx : (a == 1 ? dy : dz)) / c * (a == 0 ? 1.0 : fy);
        best = std::min(best, t);
      }
    }
    return best;
  }
  void vardt() {  // mhd.f90:422-428
    const double dtmin = vardt_min() * p.cfl;
    if (dt < 0.98 * dtmin || dt > 1.02 * dtmin) dt = dtmin;
    rkt_init();
  }
  void step() {
    vardt();
    for (int k = 0; k < 3; k++) {  // evolve, mhd.f90:303-325
      calc_flux();
      calc_rhs();
      rkt_dealias(k);
      to_real();
      update_prim();
    }
    time = time + dt;
    evolve_radius(time);
  }
};

}  // namespace

extern "C" {

// params: nx, ny, nz (powers of two, ny*nz even) and the values below; returns NULL on an
// unsupported combination
void* o2_create(int nx, int ny, int nz, double gamma, int if_resis, double eta, int if_visc, double nu, double cfl,
                int if_AEB, double R0, double Ur0, int if_Hall, double di) {
  auto pow2 = [](int n) { return n >= 2 && (n & (n - 1)) == 0; };
  if (!pow2(nx) || !pow2(ny) || !pow2(nz)) return nullptr;
  Params p{nx, ny, nz, gamma, eta, nu, cfl, R0, Ur0, di, if_resis, if_visc, if_AEB, if_Hall};
  return new Solver(p);
}
void o2_destroy(void* s) { delete static_cast<Solver*>(s); }
// primitive state (rho, u, B, p) in the reference's uu(ix,iy,iz,1:8) order; time t0 (the
// restart path: evolve_radius(t0), conserve, forward transform)
void o2_set_state(void* h, const double* prim, double t0) {
  Solver* s = static_cast<Solver*>(h);
  s->time = t0;
  s->dt = 0.0;
  s->evolve_radius(t0);
  s->set_primitive(prim);
}
void o2_step(void* h, int n, double* time, double* dt) {
  Solver* s = static_cast<Solver*>(h);
  for (int i = 0; i < n; i++) s->step();
  if (time) *time = s->time;
  if (dt) *dt = s->dt;
}
// the conserved real state uu(:,:,:,1:8) as the last stage left it
void o2_get_state(void* h, double* uu) {
  Solver* s = static_cast<Solver*>(h);
  std::memcpy(uu, s->uu.data(), sizeof(double) * 8 * s->nr);
}
int o2_threads() { return omp_get_max_threads(); }

}  // extern "C"
