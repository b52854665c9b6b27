// Host side of the engine: parameter checks, device allocation, tables, kernel dispatch
// over the supported line lengths, the fused step (captured once into a CUDA graph and
// replayed), transforms for upload / download, and diagnostics.
#pragma once
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include <chrono>
#include <cudaTypedefs.h>
#include <thread>
#include <map>
#include <array>
#include <complex>
#include "launch.cuh"
#include "diag.cuh"
#include "ic.cuh"
#include "stats.cuh"

namespace laps {


// ---------------------------------------------------------------------------- host conversions
template <class T> T host_cvt(long double x);
template <> inline double host_cvt<double>(long double x) { return (double)x; }
template <> inline float host_cvt<float>(long double x) { return (float)x; }
template <> inline dd host_cvt<dd>(long double x) {
  float h = (float)x;
  float l = (float)(x - (long double)h);
  return {h, l};
}
template <class T> typename Store<T>::C host_cplx(long double re, long double im);
template <> inline double2 host_cplx<double>(long double re, long double im) { return make_double2((double)re, (double)im); }
template <> inline float2 host_cplx<float>(long double re, long double im) { return make_float2((float)re, (float)im); }
template <> inline float4 host_cplx<dd>(long double re, long double im) {
  dd a = host_cvt<dd>(re), b = host_cvt<dd>(im);
  return make_float4(a.hi, a.lo, b.hi, b.lo);
}

// exp(-2 pi i j / n), j = 0..n-1
template <class T> std::vector<typename Store<T>::C> twiddles(int n) {
  std::vector<typename Store<T>::C> t(n);
  const long double pi = 3.141592653589793238462643383279502884L;
  for (int j = 0; j < n; j++) {
    long double a = 2.0L * pi * (long double)j / (long double)n;
    t[j] = host_cplx<T>(cosl(a), -sinl(a));
  }
  return t;
}

// A work buffer of nfields fields seen by the tile copies: 8-byte elements, dim 0 = kx
// (kxp * ew elements, ew = complex bytes / 8), dim 1 = y, dim 2 = z + field * nz; box
// {TX * ew, by, bz}.
inline CUtensorMap work_tensor_map(void* base, const Geo& g, int nfields, int ew, int by, int bz) {
  CUtensorMap m;
  cuuint64_t dims[3] = {(cuuint64_t)g.kxp * ew, (cuuint64_t)g.ny, (cuuint64_t)g.nz * nfields};
  cuuint64_t strides[2] = {(cuuint64_t)g.kxp * ew * 8, (cuuint64_t)g.ny * g.kxp * ew * 8};
  cuuint32_t box[3] = {(cuuint32_t)(TX * ew), (cuuint32_t)by, (cuuint32_t)bz};
  cuuint32_t es[3] = {1, 1, 1};
  CUresult r = tensor_map_encoder()(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, base, dims, strides, box, es,
                                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw Error{LAPS_ECUDA, "tensor map encoding failed (" + std::to_string((int)r) + ")"};
  return m;
}

// a device allocation for the duration of one call, freed on every way out of it.  Both
// the allocation and the free are ordered on the call's stream (cudaMallocAsync /
// cudaFreeAsync), so a call that gives up on a bounded wait returns at once: the free waits
// on the device for the kernels still using the buffer instead of blocking the host.
template <class X> struct DevTmp {
  X* p = nullptr;
  cudaStream_t s;
  DevTmp(size_t n, cudaStream_t stream) : s(stream) { LAPS_CK(cudaMallocAsync((void**)&p, n * sizeof(X), s)); }
  ~DevTmp() { if (p) cudaFreeAsync(p, s); }
  DevTmp(const DevTmp&) = delete;
  DevTmp& operator=(const DevTmp&) = delete;
};

class EngineBase {
 public:
  virtual ~EngineBase() {}
  virtual void upload(const double* h, int layout) = 0;
  virtual void set_time(double t) = 0;
  virtual double vardt() = 0;
  virtual void step(int n, double* time, double* dt, int* status) = 0;
  virtual void rk_stage(int irk) = 0;
  virtual void download(double* uu, double* prim) = 0;
  virtual void download_spectral(double* uf) = 0;
  virtual void upload_spectral(const double* uf) = 0;
  virtual void diagnostics(laps_diag* d) = 0;
  virtual void spectrum(int nshell, double* eu, double* eb) = 0;
  virtual void wait(int timeout_ms) = 0;
  virtual void get_time(double* t, double* dt) = 0;
  virtual void info(laps_info* i) = 0;
  virtual void step_profiled(int n, double* pass_ms, double* total_ms, int* status) = 0;
  // pieces of step() for ensembles, which enqueue several engines' steps into one graph
  virtual cudaStream_t get_stream() const = 0;
  virtual bool has_state() const = 0;
  virtual bool needs_first_step() const = 0;  // the unpruned first step after an upload
  virtual void reset_flags() = 0;             // clear status and halt (enqueued)
  virtual void enqueue_one_step() = 0;        // one step, enqueued on get_stream()
  virtual void host_state(double* time, double* dt, int* status) = 0;  // waits, then reads
  // the real state in the reference's order on the device (enqueued): 8 conserved fields at
  // the returned pointer, then u_x, u_y, u_z, p (4 fields); valid until the next call
  virtual const double* stage_real_state() = 0;
  virtual long long grid_points() const = 0;
  virtual int variant() const = 0;
  virtual const laps_params& params() const = 0;
  // device-side exchange with a caller (the closure): the 8 conserved real fields into a
  // device buffer; U += scale * duf (reference spectral layout, 8 fields) then the dealias
  virtual void set_schedule(int bits) = 0;
  virtual int schedule() const = 0;
  virtual int schedule_changes() const = 0;
  virtual void state_real_device(double* dst) = 0;
  virtual void add_spectral_device(const double* duf, double scale) = 0;
  // granular, unfused path (bisection against the reference's subroutines)
  virtual void calc_flux(double* host, int spectral) = 0;
  virtual void calc_rhs(double* host) = 0;
  virtual void dealias_state() = 0;
  // fresh-start initial conditions generated on the device (phases of ipert 6 / 7 given)
  virtual void init_fields(const laps_ic& ic, const double* phases) = 0;
  // perpendicular angle statistics of increments along one axis (4 arrays of n_axis)
  virtual void angle_statistics(int axis, double* out) = 0;
};

// T: compute type of the transforms and products; TS: storage type of the state, the RK
// register, the CFL arithmetic and the diagnostics (equal except in the FP32-transform mode)
template <class T, class TS = T> class Engine : public EngineBase {
  using C = typename Store<T>::C;
  using SR = typename Store<T>::R;
  using CS = typename Store<TS>::C;
  using SRS = typename Store<TS>::R;

 public:
  laps_params p;
  Geo gfull, gprune;
  Phys P;
  PT<T> pc;
  PT<TS> ps;
  bool prune_ok = false;   // dealias option 1: the box |k_i| <= n_i/3 holds every non-zero mode
  bool dealiased = false;  // the state has been through at least one RK stage since upload
  bool have_state = false;
  int dev = 0;
  cudaStream_t stream = nullptr;
  cudaGraphExec_t graph_steady = nullptr;
  // execution schedule (LAPS_SCHED_* bits) and the number of times it changed (an ensemble
  // recaptures its graph when a member's count moves)
  int sched = 0, sched_changes = 0;
  long long bytes = 0;
  std::vector<void*> allocs;
  Bufs<T, TS> B{};
  C *twx = nullptr, *twy = nullptr, *twz = nullptr;      // twiddles in T (passes)
  CS *twxs = nullptr, *twys = nullptr, *twzs = nullptr;  // twiddles in TS (state transforms)
  // FP32 transforms with an FP64 state: the per-field state transforms of upload and download
  // run in float-float on the FP32 pipes (48-bit significand; native FP64 transforms are
  // FP64-pipe bound, ~7x slower here), with the values converted at both ends
  static constexpr bool XDD = std::is_same<T, float>::value && std::is_same<TS, double>::value;
  float4 *twxd = nullptr, *twyd = nullptr, *twzd = nullptr;  // float-float twiddles (XDD)
  SRS *s_wx, *s_kxd, *s_wy, *s_kyd, *s_kzd, *s_kx2, *s_ky2, *s_kz2, *s_fx = nullptr, *s_fy = nullptr, *s_fz = nullptr;
  SR *t_wx, *t_kxd, *t_wy, *t_kyd, *t_kzd, *t_kx2, *t_ky2, *t_kz2, *t_fx = nullptr, *t_fy = nullptr, *t_fz = nullptr;
  double *d_wx, *d_wy, *d_wz;
  short* kxlim = nullptr;
  StepState* st = nullptr;
  StepState* h_st = nullptr;  // pinned mirror
  double* d_part = nullptr;   // diagnostics partial sums
  CUtensorMap tm_d{}, tm_e{};  // tile copies of pass D (y columns of W1) and E (z columns of W2)
  // pass A: kept kz rows of the z columns of the state U; pass B: kept ky rows of the y
  // columns of W1.  Index 0 for the whole spectrum, 1 for the pruned one: the box height of
  // each map is that geometry's KeptCopies box, which the kernel recomputes from its Geo.
  CUtensorMap tm_a[2]{}, tm_b[2]{};
  int box_a[2]{}, box_b[2]{};
  // pass E: the W2 map, then the state U and the RK register R in kept-kz boxes (L2 prefetch)
  CUtensorMap tm_e3[2][3]{};
  int box_e[2]{};
  int npart = 0;

  template <class X> X* dalloc(size_t n) {
    void* ptr = nullptr;
    LAPS_CK(cudaMalloc(&ptr, n * sizeof(X)));
    allocs.push_back(ptr);
    return (X*)ptr;
  }

  static int w2_fields(const laps_params& q) { return q.variant == LAPS_VARIANT_3DI ? 19 : 15; }
  // work buffers also stage state-type data (upload, download, diagnostics)
  static constexpr long long WE = sizeof(C) > sizeof(CS) ? sizeof(C) : sizeof(CS);
  static long long plan_bytes(const laps_params& q) {
    long long kxp = ((q.nx / 2 + 1) + 7) / 8 * 8;
    long long fsc = kxp * q.ny * q.nz;
    return 8 * fsc * ((long long)sizeof(CS) + (long long)sizeof(C)) + (19 + w2_fields(q)) * fsc * WE + (1 << 20);
  }
  template <class X> static PT<X> make_pt(const Phys& P) {
    PT<X> c;
    c.gamma = host_cvt<X>(P.gamma); c.gm1 = host_cvt<X>(P.gamma - 1.0);
    c.cg = host_cvt<X>(-2.0 * P.gamma / (P.gamma - 1.0));
    c.di = host_cvt<X>(P.di); c.nu = host_cvt<X>(P.nu); c.eta = host_cvt<X>(P.eta);
    c.cosc = host_cvt<X>(P.cos_cor); c.sinc = host_cvt<X>(P.sin_cor);
    c.inv_mindx = host_cvt<X>(1.0 / P.mindx);
    c.half = host_cvt<X>(0.5); c.two = host_cvt<X>(2.0); c.one = host_cvt<X>(1.0);
    c.zero = host_cvt<X>(0.0); c.four = host_cvt<X>(4.0);
    c.is2 = host_cvt<X>(0.70710678118654752440L);
    c.dx = host_cvt<X>(P.dx); c.dy = host_cvt<X>(P.dy); c.dz = host_cvt<X>(P.dz);
    c.eta_dx = host_cvt<X>(P.eta / P.dx); c.eta_dy = host_cvt<X>(P.eta / P.dy);
    return c;
  }

  explicit Engine(const laps_params& q) : p(q) {
    dev = q.device;
    LAPS_CK(cudaSetDevice(dev));
    Geo g{};
    g.nx = q.nx; g.ny = q.ny; g.nz = q.nz; g.nh = q.nx / 2 + 1;
    g.kxp = (g.nh + 7) / 8 * 8;
    g.fsc = (long long)g.kxp * g.ny * g.nz;
    g.fsr = (long long)g.nx * g.ny * g.nz;
    g.kx_keep = g.nh; g.ky_lo = g.ny; g.ky_hi = g.ny; g.kz_lo = g.nz; g.kz_hi = g.nz;
    gfull = g;
    // physics scalars
    const double pi = 3.141592653589793;
    P = Phys{};
    P.gamma = q.adiabatic_index;
    P.nu = q.viscosity; P.eta = q.resistivity; P.di = q.ion_inertial_length; P.cfl = q.cfl;
    P.dx = q.Lx / q.nx; P.dy = q.Ly / q.ny; P.dz = q.Lz / q.nz;
    const bool two_d = q.variant == LAPS_VARIANT_2DC, incomp = q.variant == LAPS_VARIANT_3DI;
    P.mindx = two_d ? std::fmin(P.dx, P.dy) : std::fmin(std::fmin(P.dx, P.dy), P.dz);
    P.R0 = q.radius0;
    P.Ur = q.if_AEB ? q.Ur0 : 0.0;  // mhd.f90:88-90
    double ang = q.if_corotating ? q.corotating_angle : 0.0;  // AEBmod.f90:28-30
    P.cos_cor = std::cos(ang); P.sin_cor = std::sin(ang);
    P.visc = q.if_visc; P.visc_exp = q.if_visc_exp; P.resis = q.if_resis; P.resis_exp = q.if_resis_exp;
    P.cons_bg = q.if_conserve_background; P.aeb = q.if_AEB; P.corot = q.if_AEB && q.if_corotating;
    P.hall = q.if_Hall;
    P.dealias = (q.dealias_option == 1 || q.dealias_option == 2 || (two_d && q.dealias_option == 3)) ? q.dealias_option : 0;
    P.variant = q.variant; P.two_d = two_d; P.zrad = two_d && q.if_AEB && q.if_z_radial;
    P.limit_dt = two_d && q.if_limit_dt_increase; P.dstep = two_d ? q.dstep_calcdt : 1;
    pc = make_pt<T>(P);
    ps = make_pt<TS>(P);
    // expansion damping of each variable: mhdrhs.f90:237-247; 2D/mhdrhs.f90:319-343 (radial z);
    // src_incompressible/mhdrhs.f90:187-204 (p decays with 2 gamma)
    double ebm[8] = {2.0, 2.0, 3.0, 3.0, 2.0, 1.0, 1.0, 0.0};
    if (P.zrad) { double zr[8] = {2.0, 3.0, 3.0, 2.0, 1.0, 1.0, 2.0, 0.0}; std::memcpy(ebm, zr, sizeof ebm); }
    if (incomp) ebm[7] = 2.0 * P.gamma;
    P.ebm_mask = incomp ? 0xFF : 0x7F;
    for (int v = 0; v < 8; v++) {
      pc.ebm[v] = host_cvt<T>(ebm[v]);
      ps.ebm[v] = host_cvt<TS>(ebm[v]);
    }

    // wave numbers, mhdinit.f90:88-115 (the Nyquist index takes +k)
    auto wn = [&](int n, double L) {
      std::vector<double> w(n);
      for (int i = 1; i <= n; i++) w[i - 1] = (i <= n / 2 + 1) ? 2 * pi * (i - 1) / L : 2 * pi * (i - 1 - n) / L;
      return w;
    };
    std::vector<double> wx = wn(q.nx, q.Lx), wy = wn(q.ny, q.Ly), wz = wn(q.nz, q.Lz);
    wx.resize(g.nh);

    // dealias option 1: kept kx count per (kz, ky) row with the reference's own formula
    // (dealiasing.f90:87-99), and the box that holds every kept mode
    std::vector<short> lim;
    if (P.dealias == 1 || P.dealias == 3) {
      lim.assign((size_t)q.nz * q.ny, 0);
      int kxk = 0, kyk = 0, kzk = 0;
      for (int iz = 0; iz < q.nz; iz++)
        for (int iy = 0; iy < q.ny; iy++) {
          int cnt = 0;
          for (int ix = 0; ix < g.nh; ix++) {
            double rx = wx[ix] * q.Lx / (2 * pi * q.nx), ry = wy[iy] * q.Ly / (2 * pi * q.ny);
            bool drop;
            if (two_d && P.dealias == 3)  // square truncation, 2D/dealiasing.f90:102-117
              drop = std::fabs(rx) > 1.0 / 3.0 || std::fabs(ry) > 1.0 / 3.0;
            else if (two_d)  // circle, 2D/dealiasing.f90:87-99
              drop = std::sqrt(std::pow(rx, 2) + std::pow(ry, 2)) > 1.0 / 3.0;
            else  // sphere, dealiasing.f90:87-99
              drop = std::sqrt(std::pow(rx, 2) + std::pow(ry, 2) + std::pow(wz[iz] * q.Lz / (2 * pi * q.nz), 2)) > 1.0 / 3.0;
            if (!drop) {
              if (cnt != ix) throw Error{LAPS_EINVAL, "dealias mask is not monotone in kx"};
              cnt = ix + 1;
              int my = iy <= q.ny / 2 ? iy : q.ny - iy, mz = iz <= q.nz / 2 ? iz : q.nz - iz;
              kxk = std::max(kxk, ix);
              kyk = std::max(kyk, my);
              kzk = std::max(kzk, mz);
            }
          }
          lim[(size_t)iz * q.ny + iy] = (short)cnt;
        }
      Geo gp = g;
      gp.kx_keep = kxk + 1;
      if (2 * kyk + 1 < q.ny) { gp.ky_lo = kyk + 1; gp.ky_hi = q.ny - kyk; }
      if (2 * kzk + 1 < q.nz) { gp.kz_lo = kzk + 1; gp.kz_hi = q.nz - kzk; }
      gprune = gp;
      prune_ok = true;
    } else {
      gprune = g;
    }

    LAPS_CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    side_ready();  // before any capture of the step
    B.U = dalloc<CS>(8 * g.fsc);
    B.R = dalloc<C>(8 * g.fsc);
    B.W1 = (C*)dalloc<unsigned char>(19 * g.fsc * WE);
    B.W2 = (C*)dalloc<unsigned char>(w2_fields(q) * g.fsc * WE);
    bytes = plan_bytes(q) - (1 << 20);
    {
      const int ew = (int)(sizeof(C) / 8);
      tm_d = work_tensor_map(B.W1, g, 19, ew, std::min(q.ny, 256), 1);
      tm_e = work_tensor_map(B.W2, g, w2_fields(q), ew, 1, std::min(q.nz, 256));
      for (int i = 0; i < 2; i++) {
        const Geo& gk = i ? gprune : gfull;
        box_a[i] = KeptCopies(gk.kz_lo, gk.kz_hi, q.nz, tile_gran((int)sizeof(CS))).box;
        box_b[i] = KeptCopies(gk.ky_lo, gk.ky_hi, q.ny, tile_gran((int)sizeof(C))).box;
        tm_a[i] = work_tensor_map(B.U, g, 8, (int)(sizeof(CS) / 8), 1, box_a[i]);
        tm_b[i] = work_tensor_map(B.W1, g, 19, ew, box_b[i], 1);
        box_e[i] = KeptCopies(gk.kz_lo, gk.kz_hi, q.nz, 1).box;
        tm_e3[i][0] = tm_e;
        tm_e3[i][1] = work_tensor_map(B.U, g, 8, (int)(sizeof(CS) / 8), 1, box_e[i]);
        tm_e3[i][2] = work_tensor_map(B.R, g, 8, ew, 1, box_e[i]);
      }
    }
    LAPS_CK(cudaMemsetAsync(B.U, 0, 8 * g.fsc * sizeof(CS), stream));
    LAPS_CK(cudaMemsetAsync(B.R, 0, 8 * g.fsc * sizeof(C), stream));
    auto up = [&](auto* dst, const auto& src) {
      LAPS_CK(cudaMemcpy(dst, src.data(), src.size() * sizeof(src[0]), cudaMemcpyHostToDevice));
    };
    auto twx_h = twiddles<T>(q.nx), twy_h = twiddles<T>(q.ny), twz_h = twiddles<T>(q.nz);
    twx = dalloc<C>(q.nx); up(twx, twx_h);
    twy = dalloc<C>(q.ny); up(twy, twy_h);
    twz = dalloc<C>(q.nz); up(twz, twz_h);
    auto twxs_h = twiddles<TS>(q.nx), twys_h = twiddles<TS>(q.ny), twzs_h = twiddles<TS>(q.nz);
    twxs = dalloc<CS>(q.nx); up(twxs, twxs_h);
    twys = dalloc<CS>(q.ny); up(twys, twys_h);
    twzs = dalloc<CS>(q.nz); up(twzs, twzs_h);
    if constexpr (XDD) {
      auto twxd_h = twiddles<dd>(q.nx), twyd_h = twiddles<dd>(q.ny), twzd_h = twiddles<dd>(q.nz);
      twxd = dalloc<float4>(q.nx); up(twxd, twxd_h);
      twyd = dalloc<float4>(q.ny); up(twyd, twyd_h);
      twzd = dalloc<float4>(q.nz); up(twzd, twzd_h);
    }
    d_wx = dalloc<double>(g.nh); up(d_wx, wx);
    d_wy = dalloc<double>(q.ny); up(d_wy, wy);
    d_wz = dalloc<double>(q.nz); up(d_wz, wz);
    t_wx = dalloc<SR>(g.nh); t_kxd = dalloc<SR>(g.nh); t_kx2 = dalloc<SR>(g.nh);
    t_wy = dalloc<SR>(q.ny); t_kyd = dalloc<SR>(q.ny); t_ky2 = dalloc<SR>(q.ny);
    t_kzd = dalloc<SR>(q.nz); t_kz2 = dalloc<SR>(q.nz);
    s_wx = dalloc<SRS>(g.nh); s_kxd = dalloc<SRS>(g.nh); s_kx2 = dalloc<SRS>(g.nh);
    s_wy = dalloc<SRS>(q.ny); s_kyd = dalloc<SRS>(q.ny); s_ky2 = dalloc<SRS>(q.ny);
    s_kzd = dalloc<SRS>(q.nz); s_kz2 = dalloc<SRS>(q.nz);
    if (P.dealias == 1 || P.dealias == 3) { kxlim = dalloc<short>(lim.size()); up(kxlim, lim); }
    if (P.dealias == 2) {  // dealiasing.f90:31-65
      auto filt = [&](auto tag, const std::vector<double>& w, double L, int n, double af) {
        using X = decltype(tag);
        using XR = typename Store<X>::R;
        double aj = (5.0 + 6.0 * af) / 8.0, bj = (1.0 + 2.0 * af) / 2.0, cj = -(1.0 - 2 * af) / 8.0;
        std::vector<XR> f(w.size());
        for (size_t i = 0; i < w.size(); i++) {
          double wl = w[i] * L / n;
          double v = (aj + bj * std::cos(wl) + cj * std::cos(2 * wl)) / (1 + 2 * af * std::cos(wl));
          X tv = host_cvt<X>(v);
          std::memcpy(&f[i], &tv, sizeof(XR));
        }
        return f;
      };
      auto fx = filt(T{}, wx, q.Lx, q.nx, q.afx), fy = filt(T{}, wy, q.Ly, q.ny, q.afy), fz = filt(T{}, wz, q.Lz, q.nz, q.afz);
      t_fx = dalloc<SR>(fx.size()); up(t_fx, fx);
      t_fy = dalloc<SR>(fy.size()); up(t_fy, fy);
      t_fz = dalloc<SR>(fz.size()); up(t_fz, fz);
      auto gx = filt(TS{}, wx, q.Lx, q.nx, q.afx), gy = filt(TS{}, wy, q.Ly, q.ny, q.afy), gz = filt(TS{}, wz, q.Lz, q.nz, q.afz);
      s_fx = dalloc<SRS>(gx.size()); up(s_fx, gx);
      s_fy = dalloc<SRS>(gy.size()); up(s_fy, gy);
      s_fz = dalloc<SRS>(gz.size()); up(s_fz, gz);
    }
    if ((P.dealias == 1 || P.dealias == 3) && !kxlim) throw Error{LAPS_EINVAL, "dealias table missing"};
    if (P.dealias == 2 && !(t_fx && t_fy && t_fz)) throw Error{LAPS_EINVAL, "dealias filters missing"};
    st = dalloc<StepState>(1);
    LAPS_CK(cudaMallocHost(&h_st, sizeof(StepState)));
    StepState s0{};
    s0.time = 0.0; s0.dt = 0.0; s0.radius = q.radius0;
    s0.inv_tau = P.Ur != 0.0 ? 1.0 / (q.radius0 / P.Ur) : 0.0;
    s0.r_ratio = 1.0;  // radius0 / radius at start; the factor itself is (k R0)/R below
    s0.cfl_bits = 0x7FF0000000000000ull;
    s0.cfl32_bits = 0x7F800000u;
    s0.ksq_plain = 1;  // grid_initialize's k^2 until the first evolve_radius
    s0.rho0 = q.rho0 > 0 ? q.rho0 : 1.0;
    s0.istep = 0;
    s0.R0 = P.R0;
    step_state_f32(s0);
    LAPS_CK(cudaMemcpy(st, &s0, sizeof(s0), cudaMemcpyHostToDevice));
    npart = 4096;
    d_part = dalloc<double>((size_t)npart * 32);
    tables();
    LAPS_CK(cudaStreamSynchronize(stream));
  }

  ~Engine() override {
    for (cudaEvent_t ev : ev_pool) cudaEventDestroy(ev);
    if (graph_steady) cudaGraphExecDestroy(graph_steady);
    for (void* a : allocs) cudaFree(a);
    if (h_st) cudaFreeHost(h_st);
    for (cudaEvent_t e : fev)
      if (e) cudaEventDestroy(e);
    if (cstream) cudaStreamDestroy(cstream);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    if (side) cudaStreamDestroy(side);
    if (stream) cudaStreamDestroy(stream);
  }

  KTab<T> ktab() const {
    KTab<T> K;
    K.wx = (const T*)t_wx; K.kxd = (const T*)t_kxd; K.wy = (const T*)t_wy; K.kyd = (const T*)t_kyd; K.kzd = (const T*)t_kzd;
    K.kx2 = (const T*)t_kx2; K.ky2 = (const T*)t_ky2; K.kz2 = (const T*)t_kz2;
    K.fx = (const T*)t_fx; K.fy = (const T*)t_fy; K.fz = (const T*)t_fz;
    K.kxlim = kxlim;
    return K;
  }

  KTab<TS> ktab_s() const {
    KTab<TS> K;
    K.wx = (const TS*)s_wx; K.kxd = (const TS*)s_kxd; K.wy = (const TS*)s_wy; K.kyd = (const TS*)s_kyd; K.kzd = (const TS*)s_kzd;
    K.kx2 = (const TS*)s_kx2; K.ky2 = (const TS*)s_ky2; K.kz2 = (const TS*)s_kz2;
    K.fx = (const TS*)s_fx; K.fy = (const TS*)s_fy; K.fz = (const TS*)s_fz;
    K.kxlim = kxlim;
    return K;
  }
  PassK<T, TS> passk() const { return PassK<T, TS>{pc, ps, ktab(), ktab_s()}; }

  void tables() {
    k_tables<T><<<1, 256, 0, stream>>>(d_wx, d_wy, d_wz, t_wx, t_kxd, t_wy, t_kyd, t_kzd, t_kx2, t_ky2, t_kz2, gfull.nh, p.ny,
                                       p.nz, p.radius0, P.zrad, st);
    LAPS_CK(cudaGetLastError());
    k_tables<TS><<<1, 256, 0, stream>>>(d_wx, d_wy, d_wz, s_wx, s_kxd, s_wy, s_kyd, s_kzd, s_kx2, s_ky2, s_kz2, gfull.nh, p.ny,
                                        p.nz, p.radius0, P.zrad, st);
    LAPS_CK(cudaGetLastError());
  }

  // ---------------------------------------------------------------- plain transforms
  // plain transforms of state-type data; the work buffers are reused as state-type arrays
  CS* W1s() const { return (CS*)B.W1; }
  CS* W2s() const { return (CS*)B.W2; }
  void col_plain(const CS* in, CS* out, int nf, int N, int dir, int jstride, int ostride, int ncol, int nouter, int sexp,
                 const CS* tw) {
    launch_col_plain<TS>(stream, in, out, gfull.fsc, nf, N, dir, jstride, ostride, ncol, nouter, sexp, tw);
  }
  void rows_r2c(const SRS* in, CS* out, long long nrows) { launch_rows_r2c<TS>(stream, p.nx, in, out, nrows, gfull.kxp, twxs); }
  void rows_c2r(const CS* in, SRS* out, long long nrows) { launch_rows_c2r<TS>(stream, p.nx, in, out, nrows, gfull.kxp, twxs); }
  // real TS fields (W1 layout, nf) -> spectrum `out` (fsc pitch)
  void forward3d(const SRS* real, CS* out, int nf) {
    const Geo& g = gfull;
    CS* w2 = W2s();
    rows_r2c(real, w2, (long long)nf * g.ny * g.nz);
    for (int f = 0; f < nf; f++) {
      // y: element (f, z, y, kx): jstride = kxp, outer = z with ostride ny*kxp
      col_plain(w2 + f * g.fsc, w2 + f * g.fsc, 1, g.ny, -1, g.kxp, g.ny * g.kxp, g.nh, g.nz, -ilog2(g.ny), twys);
      // z: jstride = ny*kxp, outer = y with ostride kxp
      col_plain(w2 + f * g.fsc, out + f * g.fsc, 1, g.nz, -1, g.ny * g.kxp, g.kxp, g.nh, g.ny, -ilog2(g.nz), twzs);
    }
  }
  // spectrum (nf fields) -> real TS fields in W1
  void inverse3d(const CS* spec, int nf) {
    const Geo& g = gfull;
    CS* w2 = W2s();
    for (int f = 0; f < nf; f++) {
      col_plain(spec + f * g.fsc, w2 + f * g.fsc, 1, g.nz, +1, g.ny * g.kxp, g.kxp, g.nh, g.ny, 0, twzs);
      col_plain(w2 + f * g.fsc, w2 + f * g.fsc, 1, g.ny, +1, g.kxp, g.ny * g.kxp, g.nh, g.nz, 0, twys);
    }
    rows_c2r(w2, (SRS*)B.W1, (long long)nf * g.ny * g.nz);
  }

  // ---------------------------------------------------------------- fused passes
  PassArgs args(const Geo& g, int stage, int store_rk, int cfl) {
    PassArgs a;
    a.g = g; a.P = P; a.hall = P.hall; a.aeb = P.aeb; a.stage = stage; a.store_rk = store_rk; a.cfl = cfl; a.st = st;
    a.mass_from_state = P.variant != LAPS_VARIANT_3DI && (P.dealias == 1 || P.dealias == 3);
    a.e_first = 0;
    a.rhs_only = rhs_mode;
    a.mass_done = 0;
    a.sched = sched;
    return a;
  }
  // the map whose box matches the kept-row copies the kernel makes for a.g
  const CUtensorMap* kept_map(const CUtensorMap* m, const int* box, int want) const {
    if (box[1] == want) return &m[1];
    if (box[0] == want) return &m[0];
    throw Error{LAPS_EINVAL, "no tile map for this geometry"};
  }
  void passA(const PassArgs& a) {
    launch_passA<T, TS>(stream, p.nz, B, a, passk(), twz, kept_map(tm_a, box_a, KeptCopies(a.g.kz_lo, a.g.kz_hi, p.nz, tile_gran((int)sizeof(CS))).box));
  }
  void passB(const PassArgs& a) {
    launch_passB<T, TS>(stream, p.ny, B, a, passk(), twy, kept_map(tm_b, box_b, KeptCopies(a.g.ky_lo, a.g.ky_hi, p.ny, tile_gran((int)sizeof(C))).box));
  }
  void passC(const PassArgs& a) { launch_passC<T, TS>(stream, p.nx, B, a, passk(), twx); }
  void passD(const PassArgs& a) { launch_passD<T, TS>(stream, p.ny, B, a, passk(), twy, &tm_d); }
  void passE(const PassArgs& a) {
    if (P.variant == LAPS_VARIANT_3DI) launch_passE3i<T, TS>(stream, p.nz, B, a, passk(), twz, nullptr);
    else {
      const int want = KeptCopies(a.g.kz_lo, a.g.kz_hi, p.nz, 1).box;
      const int i = box_e[1] == want ? 1 : 0;
      if (box_e[i] != want) throw Error{LAPS_EINVAL, "no tile map for this geometry"};
      launch_passE<T, TS>(stream, p.nz, B, a, passk(), twz, tm_e3[i]);
    }
  }

  // geometry of the inverse side (A-C) and of the forward side (D-E) of a stage
  const Geo& g_in() const { return (prune_ok && dealiased && !force_full) ? gprune : gfull; }
  const Geo& g_out() const { return (prune_ok && !force_full) ? gprune : gfull; }
  bool rhs_mode = false;    // pass E stores fnl in R and leaves the state (calc_rhs)
  bool force_full = false;  // every pass over the whole spectrum (calc_rhs)

  // one stage: stage = 0..2; cfl: compute the CFL minimum and finalise dt before D
  void enqueue_stage(int stage, bool cfl, bool store_rk) {
    const Geo& gi = g_in();
    PassArgs ai = args(gi, stage, store_rk, cfl);
    if (!P.two_d) passA(ai);  // nz = 1: pass B reads the state directly
    mark(0);
    passB(ai);
    mark(1);
    // pass C reads the inverse-side ranges and writes the forward-side kx range
    PassArgs ac = ai;
    ac.g.kx_keep = std::max(gi.kx_keep, g_out().kx_keep);
    passC(ac);
    mark(2);
    if (cfl) {
      k_finalize_dt<<<1, 32, 0, stream>>>(st, P.cfl, P.dstep, P.limit_dt, 0);
      LAPS_CK(cudaGetLastError());
      mark(5);
    }
    PassArgs ao = args(g_out(), stage, store_rk, 0);
    // the first stage after an upload must also clear every mode outside the kept box
    if (!dealiased) ao.g = gfull;
    // the continuity update reads and writes only the state and RK register, which pass D
    // does not touch: it runs on a side stream beside pass D, joined before pass E
    const bool fork = ao.mass_from_state && !ao.rhs_only && P.variant != LAPS_VARIANT_3DI && !(sched & LAPS_SCHED_INLINE_MASS);
    if (fork) {
      side_ready();
      LAPS_CK(cudaEventRecord(ev_fork, stream));
      LAPS_CK(cudaStreamWaitEvent(side, ev_fork, 0));
      launch_mass_rk<T, TS>(side, B, ao, passk());
      LAPS_CK(cudaEventRecord(ev_join, side));
    }
    passD(ao);
    mark(3);
    if (fork) {
      LAPS_CK(cudaStreamWaitEvent(stream, ev_join, 0));
      ao.mass_done = 1;
    }
    passE(ao);
    mark(4);
    dealiased = true;
  }
  void enqueue_step() {
    enqueue_stage(0, true, true);
    enqueue_stage(1, false, true);
    enqueue_stage(2, false, false);
    k_advance_time<<<1, 32, 0, stream>>>(st, p.radius0, P.Ur, P.variant == LAPS_VARIANT_3DI);
    LAPS_CK(cudaGetLastError());
    // the wave-number tables follow the radius; without expansion (Ur = 0) R stays R0 and
    // the tables built at creation / set_time stay exact (R0 / R = 1, so k^2 = (k R0 / R)^2)
    if (P.Ur != 0.0) tables();
    mark(5);
  }

  // ---------------------------------------------------------------- profiling marks
  // When `prof_on`, an event is recorded after every kernel of the step; the time between
  // consecutive events is attributed to the kernel kind recorded with the later one.
  bool prof_on = false;
  std::vector<cudaEvent_t> ev_pool;
  std::vector<int> ev_kind;
  size_t ev_used = 0;
  void mark(int kind) {
    if (!prof_on) return;
    if (ev_used == ev_pool.size()) {
      cudaEvent_t e;
      LAPS_CK(cudaEventCreate(&e));
      ev_pool.push_back(e);
      ev_kind.push_back(0);
    }
    ev_kind[ev_used] = kind;
    LAPS_CK(cudaEventRecord(ev_pool[ev_used], stream));
    ev_used++;
  }
  void step_profiled(int n, double* pass_ms, double* total_ms, int* status) override {
    if (!have_state) throw Error{LAPS_ESTATE, "no state uploaded"};
    LAPS_CK(cudaMemsetAsync(&st->status, 0, sizeof(int), stream));
    LAPS_CK(cudaMemsetAsync(&st->halt, 0, sizeof(int), stream));
    prof_on = true;
    ev_used = 0;
    mark(-1);
    for (int i = 0; i < n; i++) enqueue_step();
    prof_on = false;
    read_state();
    for (int k = 0; k < 6; k++) pass_ms[k] = 0.0;
    for (size_t i = 1; i < ev_used; i++) {
      float ms = 0.f;
      LAPS_CK(cudaEventElapsedTime(&ms, ev_pool[i - 1], ev_pool[i]));
      pass_ms[ev_kind[i]] += ms;
    }
    float tot = 0.f;
    if (ev_used > 1) LAPS_CK(cudaEventElapsedTime(&tot, ev_pool[0], ev_pool[ev_used - 1]));
    *total_ms = tot;
    if (status) *status = h_st->status;
  }

  void wait(int timeout_ms) override {
    cudaEvent_t ev;
    LAPS_CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    LAPS_CK(cudaEventRecord(ev, stream));
    auto t0 = std::chrono::steady_clock::now();
    for (;;) {
      cudaError_t e = cudaEventQuery(ev);
      if (e == cudaSuccess) break;
      if (e != cudaErrorNotReady) {
        cudaEventDestroy(ev);
        throw Error{LAPS_ECUDA, std::string("device error: ") + cudaGetErrorString(e)};
      }
      auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::steady_clock::now() - t0).count();
      if (timeout_ms > 0 && ms > timeout_ms) {
        cudaEventDestroy(ev);
        throw Error{LAPS_ETIMEDOUT, "device work did not finish within the timeout"};
      }
      std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
    cudaEventDestroy(ev);
  }
  int tmo() const { return p.timeout_ms > 0 ? p.timeout_ms : 600000; }
  void read_state() {
    LAPS_CK(cudaMemcpyAsync(h_st, st, sizeof(StepState), cudaMemcpyDeviceToHost, stream));
    wait(tmo());
  }

  // ---------------------------------------------------------------- API
  // copies between the host and the device run on their own stream, field by field, so that
  // the transforms of the fields that have arrived (upload) or are done (download) overlap them
  cudaStream_t cstream = nullptr;
  cudaEvent_t fev[13] = {};
  // side stream of the step (the continuity update beside pass D)
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  void side_ready() {
    if (side) return;
    LAPS_CK(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
    LAPS_CK(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
    LAPS_CK(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
  }
  void copy_stream_ready() {
    if (cstream) return;
    LAPS_CK(cudaStreamCreateWithFlags(&cstream, cudaStreamNonBlocking));
    for (auto& e : fev) LAPS_CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }
  // one real field -> its spectrum through the intermediate tmp (one spectral field); the
  // float-float route (XDD) converts the real field in place, so its input is consumed
  void forward_one(const SRS* real, CS* out, CS* tmp) {
    const Geo& g = gfull;
    if constexpr (XDD) {
      float2* rd = (float2*)const_cast<SRS*>(real);
      float4* td = (float4*)tmp;
      k_f64_to_dd<<<1024, 256, 0, stream>>>((const double*)real, rd, g.fsr);
      LAPS_CK(cudaGetLastError());
      launch_rows_r2c<dd>(stream, p.nx, rd, td, (long long)g.ny * g.nz, g.kxp, twxd);
      launch_col_plain<dd>(stream, td, td, g.fsc, 1, g.ny, -1, g.kxp, g.ny * g.kxp, g.nh, g.nz, -ilog2(g.ny), twyd);
      launch_col_plain<dd>(stream, td, td, g.fsc, 1, g.nz, -1, g.ny * g.kxp, g.kxp, g.nh, g.ny, -ilog2(g.nz), twzd);
      k_dd_to_f64<<<1024, 256, 0, stream>>>((const float2*)td, (double*)out, 2 * g.fsc);
      LAPS_CK(cudaGetLastError());
      return;
    }
    rows_r2c(real, tmp, (long long)g.ny * g.nz);
    col_plain(tmp, tmp, 1, g.ny, -1, g.kxp, g.ny * g.kxp, g.nh, g.nz, -ilog2(g.ny), twys);
    col_plain(tmp, out, 1, g.nz, -1, g.ny * g.kxp, g.kxp, g.nh, g.ny, -ilog2(g.nz), twzs);
  }
  void inverse_one(const CS* spec, SRS* real, CS* tmp) {
    const Geo& g = gfull;
    if constexpr (XDD) {
      float4* td = (float4*)tmp;
      k_f64_to_dd<<<1024, 256, 0, stream>>>((const double*)spec, (float2*)td, 2 * g.fsc);
      LAPS_CK(cudaGetLastError());
      launch_col_plain<dd>(stream, td, td, g.fsc, 1, g.nz, +1, g.ny * g.kxp, g.kxp, g.nh, g.ny, 0, twzd);
      launch_col_plain<dd>(stream, td, td, g.fsc, 1, g.ny, +1, g.kxp, g.ny * g.kxp, g.nh, g.nz, 0, twyd);
      launch_rows_c2r<dd>(stream, p.nx, td, (float2*)real, (long long)g.ny * g.nz, g.kxp, twxd);
      k_dd_to_f64<<<1024, 256, 0, stream>>>((const float2*)real, (double*)real, g.fsr);
      LAPS_CK(cudaGetLastError());
      return;
    }
    col_plain(spec, tmp, 1, g.nz, +1, g.ny * g.kxp, g.kxp, g.nh, g.ny, 0, twzs);
    col_plain(tmp, tmp, 1, g.ny, +1, g.kxp, g.ny * g.kxp, g.nh, g.nz, 0, twys);
    rows_c2r(tmp, real, (long long)g.ny * g.nz);
  }

  void upload(const double* h, int layout) override {
    const Geo& g = gfull;
    copy_stream_ready();
    // the 8 float64 fields land in W2; the per-field transform works through the 9th
    // spectral field of W2, after them (8 fsr doubles <= 8 fsc state-type complexes)
    double* stage = (double*)B.W2;
    CS* tmp = W2s() + 8 * g.fsc;
    for (int f = 0; f < 8; f++) {
      LAPS_CK(cudaMemcpyAsync(stage + f * g.fsr, h + f * g.fsr, g.fsr * sizeof(double), cudaMemcpyHostToDevice, cstream));
      LAPS_CK(cudaEventRecord(fev[f], cstream));
    }
    // field f needs fields <= f (rho for the momentum, all for the energy): convert and
    // transform each as soon as it is in
    for (int f = 0; f < 8; f++) {
      LAPS_CK(cudaStreamWaitEvent(stream, fev[f], 0));
      k_upload_field<TS><<<1024, 256, 0, stream>>>(stage, (SRS*)B.W1, g.fsr, f, layout == LAPS_LAYOUT_PRIMITIVE, P.gamma,
                                                   P.variant == LAPS_VARIANT_3DI);
      LAPS_CK(cudaGetLastError());
      forward_one((const SRS*)B.W1 + f * g.fsr, B.U + f * g.fsc, tmp);
    }
    // mhd.f90:135: dt = 0 before the first vardt, so the first CFL value is taken as is
    LAPS_CK(cudaMemsetAsync(&st->dt, 0, sizeof(double), stream));
    dealiased = false;
    have_state = true;
    wait(tmo());
  }
  void init_fields(const laps_ic& ic, const double* ph) override {
    const Geo& g = gfull;
    IcDev d{};
    d.ic = ic;
    d.Lx = p.Lx; d.Ly = p.Ly; d.Lz = p.Lz;
    d.cosc = P.cos_cor; d.sinc = P.sin_cor;
    d.gamma = P.gamma;
    d.incomp = P.variant == LAPS_VARIANT_3DI;
    d.modes = ic.ipert == 6 || ic.ipert == 7;
    if (d.modes) {
      // the mode sums as half-spectrum coefficients: A cos(k.x + phi) is A/2 e^{i phi} at k
      // (and its conjugate at -k, stored explicitly on the kx = 0 plane); modes that meet
      // at one wave vector add up
      std::map<long long, std::array<std::complex<double>, 7>> acc;
      auto put = [&](int f, int ikx, int iky, int ikz, std::complex<double> c) {
        const long long yi = ((iky % p.ny) + p.ny) % p.ny, zi = ((ikz % p.nz) + p.nz) % p.nz;
        const long long key = (zi * p.ny + yi) * g.kxp + ikx;
        auto it = acc.find(key);
        if (it == acc.end()) it = acc.emplace(key, std::array<std::complex<double>, 7>{}).first;
        it->second[f] += c;
      };
      auto add = [&](int f, int ikx, int iky, int ikz, double A, double phi) {
        if (ikx < 0 || (ikx == 0 && (iky < 0 || (iky == 0 && ikz < 0)))) {
          ikx = -ikx; iky = -iky; ikz = -ikz; phi = -phi;
        }
        const std::complex<double> c = 0.5 * A * std::polar(1.0, phi);
        put(f, ikx, iky, ikz, c);
        if (ikx == 0) put(f, 0, -iky, -ikz, std::conj(c));
      };
      const double pi = 3.141592653589793, half_pi = 0.5 * pi;
      const int mx = ic.nmodex, my = ic.nmodey, mz = ic.nmodez;
      if (ic.ipert == 6) {  // mhdinit.f90:487-634: outward waves, then inward ones
        const long long nm = (long long)mx * (2 * my + 1) * (2 * mz + 1);
        const double sgn = std::copysign(1.0, ic.bx0);
        for (int w = 0; w < 2; w++) {
          const int dirx = w ? -1 : 1;
          const double su = w ? 1.0 : -1.0, io = w ? ic.in_out_ratio : 1.0;
          for (int ikx = 1; ikx <= mx; ikx++)
            for (int iky = -my; iky <= my; iky++)
              for (int ikz = -mz; ikz <= mz; ikz++) {
                const double ax = std::sqrt(1 / (double)ikx), ay = iky == 0 ? 1.0 : std::sqrt(1 / (double)std::abs(iky)),
                             az = ikz == 0 ? 1.0 : std::sqrt(1 / (double)std::abs(ikz));
                const double a = ax * ay * az * io;
                const double ph0 = ph[w * nm + ((long long)(ikx - 1) * (2 * my + 1) + iky + my) * (2 * mz + 1) + ikz + mz];
                const int kx = dirx * ikx;
                if (iky == 0 && ikz == 0) {
                  add(5, kx, 0, 0, ic.db0 * a, ph0);
                  add(6, kx, 0, 0, ic.db0 * a, ph0 - half_pi);
                  add(2, kx, 0, 0, su * sgn * ic.db0 * a, ph0);
                  add(3, kx, 0, 0, su * sgn * ic.db0 * a, ph0 - half_pi);
                } else {
                  const double ky = iky * 2 * pi / p.Ly, kz = ikz * 2 * pi / p.Lz, kk = std::sqrt(ky * ky + kz * kz);
                  const double dby = ic.db0 * kz / kk, dbz = -ic.db0 * ky / kk;
                  add(5, kx, iky, ikz, dby * a, ph0);
                  add(6, kx, iky, ikz, dbz * a, ph0);
                  add(2, kx, iky, ikz, su * sgn * dby * a, ph0);
                  add(3, kx, iky, ikz, su * sgn * dbz * a, ph0);
                }
              }
        }
      } else {  // mhdinit.f90:690-930: u, B, rho modes perpendicular to k and B0
        const long long nm = (long long)(2 * mx + 1) * (2 * my + 1) * (2 * mz + 1);
        const double corr = -0.05;
        const double B0mod = std::sqrt(ic.bx0 * ic.bx0 + ic.by0 * ic.by0 + ic.bz0 * ic.bz0);
        const int mmax = std::max(mx, std::max(my, mz));
        for (int ikx = 0; ikx <= mx; ikx++)
          for (int iky = -my; iky <= my; iky++)
            for (int ikz = -mz; ikz <= mz; ikz++) {
              if ((ikx == 0 && iky < 0) || (ikx == 0 && iky == 0 && ikz <= 0)) continue;
              const double kr = std::sqrt((double)(ikx * ikx + iky * iky + ikz * ikz));
              if (kr > mmax) continue;
              const double kx = ikx * 2 * pi / p.Lx, ky = iky * 2 * pi / p.Ly, kz = ikz * 2 * pi / p.Lz;
              const double kmod = std::sqrt(kx * kx + ky * ky + kz * kz);
              const double dv[3] = {(ky * ic.bz0 - kz * ic.by0) / kmod / B0mod, (kz * ic.bx0 - kx * ic.bz0) / kmod / B0mod,
                                    (kx * ic.by0 - ky * ic.bx0) / kmod / B0mod};
              const long long j = ((long long)(ikx + mx) * (2 * my + 1) + iky + my) * (2 * mz + 1) + ikz + mz;
              const double ph0 = ph[j], ph1 = ph[nm + j], ph2 = ph[2 * nm + j];
              const double kr3 = std::sqrt(kr * kr * kr);
              for (int c = 0; c < 3; c++) add(1 + c, ikx, iky, ikz, std::sqrt(1 - corr * corr) * ic.dv0 / kr3 * dv[c], ph0);
              for (int c = 0; c < 3; c++) add(4 + c, ikx, iky, ikz, ic.db0 / kr3 * dv[c], ph1);
              for (int c = 0; c < 3; c++) add(1 + c, ikx, iky, ikz, corr * ic.dv0 / kr3 * dv[c], ph1);
              add(0, ikx, iky, ikz, ic.drho0 / kr3, ph2);
            }
      }
      std::vector<long long> hidx;
      std::vector<double2> hval;
      for (auto& kv : acc) {
        hidx.push_back(kv.first);
        for (int f = 0; f < 7; f++) hval.push_back(make_double2(kv.second[f].real(), kv.second[f].imag()));
      }
      LAPS_CK(cudaMemsetAsync(B.U, 0, 7 * g.fsc * sizeof(CS), stream));
      const int cnt = (int)hidx.size();
      if (cnt > 0) {
        DevTmp<long long> didx(hidx.size(), stream);
        DevTmp<double2> dval(hval.size(), stream);
        LAPS_CK(cudaMemcpyAsync(didx.p, hidx.data(), hidx.size() * sizeof(long long), cudaMemcpyHostToDevice, stream));
        LAPS_CK(cudaMemcpyAsync(dval.p, hval.data(), hval.size() * sizeof(double2), cudaMemcpyHostToDevice, stream));
        k_place_modes<TS><<<(cnt + 255) / 256, 256, 0, stream>>>(B.U, g.fsc, didx.p, dval.p, cnt);
        LAPS_CK(cudaGetLastError());
        wait(tmo());
      }
      inverse3d(B.U, 7);  // the mode sums on the grid: W1 real fields 0..6
    }
    k_init_fields<TS><<<1024, 256, 0, stream>>>((SRS*)B.W1, g, d);
    LAPS_CK(cudaGetLastError());
    forward3d((const SRS*)B.W1, B.U, 8);
    LAPS_CK(cudaMemsetAsync(&st->dt, 0, sizeof(double), stream));
    dealiased = false;
    have_state = true;
    wait(tmo());
  }
  void set_time(double t) override {
    read_state();  // sync mirror
    StepState s = *h_st;
    s.time = t;
    s.radius = p.radius0 + P.Ur * t;
    s.inv_tau = P.Ur != 0.0 ? 1.0 / (s.radius / P.Ur) : 0.0;
    s.r_ratio = p.radius0 / s.radius;
    s.ksq_plain = 0;
    step_state_f32(s);
    LAPS_CK(cudaMemcpyAsync(st, &s, sizeof(s), cudaMemcpyHostToDevice, stream));
    tables();
    wait(tmo());
  }
  double vardt() override {
    if (!have_state) throw Error{LAPS_ESTATE, "no state uploaded"};
    const Geo& gi = g_in();
    PassArgs a = args(gi, 0, 0, 1);
    if (!P.two_d) passA(a);
    passB(a);
    PassArgs ac = a;
    ac.cfl = 2;  // CFL only: skip the fluxes
    passC(ac);
    k_finalize_dt<<<1, 32, 0, stream>>>(st, P.cfl, P.dstep, P.limit_dt, 1);
    LAPS_CK(cudaGetLastError());
    read_state();
    return h_st->dt;
  }
  cudaStream_t get_stream() const override { return stream; }
  bool has_state() const override { return have_state; }
  bool needs_first_step() const override { return !dealiased; }
  void reset_flags() override {
    LAPS_CK(cudaMemsetAsync(&st->status, 0, sizeof(int), stream));
    LAPS_CK(cudaMemsetAsync(&st->halt, 0, sizeof(int), stream));
  }
  void enqueue_one_step() override { enqueue_step(); }
  void host_state(double* time, double* dt, int* status) override {
    read_state();
    if (time) *time = h_st->time;
    if (dt) *dt = h_st->dt;
    if (status) *status = h_st->status;
  }

  void step(int n, double* time, double* dt, int* status) override {
    if (!have_state) throw Error{LAPS_ESTATE, "no state uploaded"};
    LAPS_CK(cudaMemsetAsync(&st->status, 0, sizeof(int), stream));
    LAPS_CK(cudaMemsetAsync(&st->halt, 0, sizeof(int), stream));
    int done = 0;
    if (!dealiased && n > 0) {  // first step after an upload runs unpruned, outside the graph
      enqueue_step();
      done = 1;
    }
    if (done < n) {
      if (!graph_steady) {
        cudaGraph_t gr;
        LAPS_CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        enqueue_step();
        LAPS_CK(cudaStreamEndCapture(stream, &gr));
        LAPS_CK(cudaGraphInstantiate(&graph_steady, gr, 0));
        cudaGraphDestroy(gr);
      }
      for (; done < n; done++) LAPS_CK(cudaGraphLaunch(graph_steady, stream));
    }
    read_state();
    if (time) *time = h_st->time;
    if (dt) *dt = h_st->dt;
    if (status) *status = h_st->status;
  }
  void rk_stage(int irk) override {
    if (!have_state) throw Error{LAPS_ESTATE, "no state uploaded"};
    if (irk < 1 || irk > 3) throw Error{LAPS_EINVAL, "irk must be 1, 2 or 3"};
    LAPS_CK(cudaMemsetAsync(&st->halt, 0, sizeof(int), stream));
    enqueue_stage(irk - 1, false, true);
    wait(tmo());
  }
  const double* stage_real_state() override {
    if (!have_state) throw Error{LAPS_ESTATE, "no state uploaded"};
    const Geo& g = gfull;
    inverse3d(B.U, 8);
    double* out = (double*)B.W2;  // 12 real float64 fields fit in 15 complex fields
    k_download_convert<TS><<<1024, 256, 0, stream>>>((const SRS*)B.W1, out, out + 8 * g.fsr, g.fsr, P.gamma,
                                                     P.variant == LAPS_VARIANT_3DI);
    LAPS_CK(cudaGetLastError());
    return out;
  }
  void set_schedule(int bits) override {
    if (bits < 0 || bits > LAPS_SCHED_ALL) throw Error{LAPS_EINVAL, "unknown schedule bits"};
    if (bits == sched) return;
    wait(tmo());
    sched = bits;
    sched_changes++;
    if (graph_steady) {  // the captured step holds the previous schedule
      cudaGraphExecDestroy(graph_steady);
      graph_steady = nullptr;
    }
  }
  int schedule() const override { return sched; }
  int schedule_changes() const override { return sched_changes; }
  void state_real_device(double* dst) override {
    const double* rs = stage_real_state();
    LAPS_CK(cudaMemcpyAsync(dst, rs, 8 * gfull.fsr * sizeof(double), cudaMemcpyDeviceToDevice, stream));
    wait(tmo());
  }
  void add_spectral_device(const double* duf, double scale) override {
    if (!have_state) throw Error{LAPS_ESTATE, "no state uploaded"};
    k_spec_axpy_ref<TS><<<1024, 256, 0, stream>>>((const double2*)duf, B.U, gfull, 8, scale);
    LAPS_CK(cudaGetLastError());
    dealias_state();  // (waits)
  }
  void angle_statistics(int axis, double* hout) override {
    const double* rs = stage_real_state();  // 8 conserved fields, then ux, uy, uz, p
    const Geo& g = gfull;
    const int naxis = axis == 0 ? p.nx : (axis == 1 ? p.ny : p.nz);
    const int nl = naxis / 2;
    std::memset(hout, 0, 4 * (size_t)naxis * sizeof(double));
    if (nl < 1) return;
    const int nblk = (int)std::min<long long>(4 * 152, (g.fsr + ANG_THREADS - 1) / ANG_THREADS);
    DevTmp<double> dmean(4, stream), dout(4 * (size_t)naxis, stream), part((size_t)nl * nblk * ANG_NSUM, stream);
    k_state_means<TS><<<1, 32, 0, stream>>>(B.U, g.fsc, dmean.p);
    LAPS_CK(cudaGetLastError());
    double m[4];
    LAPS_CK(cudaMemcpyAsync(m, dmean.p, sizeof(m), cudaMemcpyDeviceToHost, stream));
    wait(tmo());
    // statistics.c:86-101: b0 = <B> / |<B>|
    const double b0abs = std::sqrt(m[1] * m[1] + m[2] * m[2] + m[3] * m[3]);
    AngArgs a;
    a.u = rs + 8 * g.fsr;
    a.B = rs + 4 * g.fsr;
    a.n = g.fsr;
    a.nx = p.nx; a.ny = p.ny; a.nz = p.nz; a.axis = axis; a.lag0 = 1;
    a.sqrt_rho0 = std::sqrt(m[0]);
    a.b0x = m[1] / b0abs; a.b0y = m[2] / b0abs; a.b0z = m[3] / b0abs;
    LAPS_CK(cudaMemsetAsync(dout.p, 0, 4 * (size_t)naxis * sizeof(double), stream));
    k_angle_partial<<<dim3(nblk, nl), ANG_THREADS, 0, stream>>>(a, part.p);
    LAPS_CK(cudaGetLastError());
    k_angle_final<<<(nl + 127) / 128, 128, 0, stream>>>(part.p, nblk, nl, 1, naxis, dout.p);
    LAPS_CK(cudaGetLastError());
    LAPS_CK(cudaMemcpyAsync(hout, dout.p, 4 * (size_t)naxis * sizeof(double), cudaMemcpyDeviceToHost, stream));
    wait(tmo());
  }
  const laps_params& params() const override { return p; }
  long long grid_points() const override { return gfull.fsr; }
  int variant() const override { return P.variant; }
  void download(double* uu, double* prim) override {
    if (!have_state) throw Error{LAPS_ESTATE, "no state uploaded"};
    const Geo& g = gfull;
    copy_stream_ready();
    double* out = (double*)B.W2;  // 12 real float64 fields fit in 15 complex fields
    // the per-field inverse works through one spectral field of W1 after the 8 real fields
    SRS* real = (SRS*)B.W1;
    CS* tmp = (CS*)((unsigned char*)B.W1 + (8 * g.fsr * (long long)sizeof(SRS) + 255) / 256 * 256);
    for (int f = 0; f < 8; f++) {
      inverse_one(B.U + f * g.fsc, real + f * g.fsr, tmp);
      if (uu) {  // conserved field f: convert, then copy while the next field transforms
        k_field_to_double<TS><<<1024, 256, 0, stream>>>(real + f * g.fsr, out + f * g.fsr, g.fsr);
        LAPS_CK(cudaGetLastError());
        LAPS_CK(cudaEventRecord(fev[f], stream));
        LAPS_CK(cudaStreamWaitEvent(cstream, fev[f], 0));
        LAPS_CK(cudaMemcpyAsync(uu + f * g.fsr, out + f * g.fsr, g.fsr * sizeof(double), cudaMemcpyDeviceToHost, cstream));
      }
    }
    if (prim) {  // the primitives need every field
      k_download_convert<TS><<<1024, 256, 0, stream>>>((const SRS*)real, nullptr, out + 8 * g.fsr, g.fsr, P.gamma,
                                                       P.variant == LAPS_VARIANT_3DI);
      LAPS_CK(cudaGetLastError());
      LAPS_CK(cudaEventRecord(fev[8], stream));
      LAPS_CK(cudaStreamWaitEvent(cstream, fev[8], 0));
      LAPS_CK(cudaMemcpyAsync(prim, out + 8 * g.fsr, 4 * g.fsr * sizeof(double), cudaMemcpyDeviceToHost, cstream));
    }
    LAPS_CK(cudaEventRecord(fev[12], cstream));
    LAPS_CK(cudaStreamWaitEvent(stream, fev[12], 0));
    wait(tmo());
  }
  void download_spectral(double* uf) override {
    const Geo& g = gfull;
    double2* out = (double2*)B.W1;
    k_spec_to_ref<TS><<<1024, 256, 0, stream>>>(B.U, out, g, 8);
    LAPS_CK(cudaGetLastError());
    LAPS_CK(cudaMemcpyAsync(uf, out, (size_t)8 * g.nz * g.ny * g.nh * sizeof(double2), cudaMemcpyDeviceToHost, stream));
    wait(tmo());
  }
  void upload_spectral(const double* uf) override {
    const Geo& g = gfull;
    double2* in = (double2*)B.W1;
    LAPS_CK(cudaMemcpyAsync(in, uf, (size_t)8 * g.nz * g.ny * g.nh * sizeof(double2), cudaMemcpyHostToDevice, stream));
    k_spec_from_ref<TS><<<1024, 256, 0, stream>>>(in, B.U, g, 8);
    LAPS_CK(cudaGetLastError());
    dealiased = false;
    have_state = true;
    wait(tmo());
  }
  void diagnostics(laps_diag* d) override;
  void spectrum(int nshell, double* eu, double* eb) override;
  void calc_flux(double* host, int spectral) override;
  void calc_rhs(double* host) override;
  void dealias_state() override;
  double* d_spec = nullptr;  // per-block shell partials of spectrum()
  size_t spec_cap = 0;
  void get_time(double* t, double* dt) override {
    read_state();
    if (t) *t = h_st->time;
    if (dt) *dt = h_st->dt;
  }
  void info(laps_info* i) override {
    i->device_bytes = bytes;
    i->kx_keep = gprune.kx_keep;
    i->ky_keep = gprune.nky();
    i->kz_keep = gprune.nkz();
    // per stage: passes A (3-D), B, C, D, E (E in two launches when the continuity term comes
    // from the momentum); per step: dt finalisation, time advance, two table updates
    const bool mass = P.variant != LAPS_VARIANT_3DI && (P.dealias == 1 || P.dealias == 3);
    i->kernels_per_step = 3 * ((P.two_d ? 4 : 5) + (mass ? 1 : 0)) + 2 + (P.Ur != 0.0 ? 2 : 0);
    i->graph = graph_steady != nullptr;
  }
};

// ---------------------------------------------------------------------------- granular path
// calc_flux (mhdrhs.f90:21-124) alone: the state and, with the Hall term, J = i k x B
// (calc_current_density_real, :296-362) to real space, then the fluxes one at a time, as real
// fields or (spectral != 0) forward-transformed like transform_flux_real_to_fourier
// (:128-172).  Output: nflux fields of nx*ny*nz reals, or of (nx/2+1)*ny*nz complex values.
template <class T, class TS> void Engine<T, TS>::calc_flux(double* host, int spectral) {
  if (!have_state) throw Error{LAPS_ESTATE, "no state uploaded"};
  if (P.variant == LAPS_VARIANT_3DI) throw Error{LAPS_EINVAL, "the flux entry points serve the compressible variants"};
  const Geo& g = gfull;
  read_state();
  const long long n = g.fsr;
  const int nb = 1024;
  SRS* real = (SRS*)B.W1;  // inputs: state 0..7, J 8..10
  inverse3d(B.U, 8);
  CS* w2 = W2s();
  const long long w2f = w2_fields(p) * WE / (long long)sizeof(CS);  // W2 capacity in CS fields
  CS* slot = w2 + (w2f - 1) * g.fsc;
  int nin = 8;
  if (P.hall) {
    for (int c = 0; c < 3; c++) {
      k_spec_curl<TS><<<nb, 256, 0, stream>>>(B.U, slot, g, ktab_s(), P, ps, st, c);
      LAPS_CK(cudaGetLastError());
      // one field: z then y columns in W2 field 0, then the rows into the input slot
      col_plain(slot, w2, 1, g.nz, +1, g.ny * g.kxp, g.kxp, g.nh, g.ny, 0, twzs);
      col_plain(w2, w2, 1, g.ny, +1, g.kxp, g.ny * g.kxp, g.nh, g.nz, 0, twys);
      rows_c2r(w2, real + (8 + c) * n, (long long)g.ny * g.nz);
    }
    nin = 11;
  }
  const int nflux = 18 + (P.aeb ? 1 : 0);
  const long long nspec = (long long)g.nz * g.ny * g.nh;
  for (int k = 0; k < nflux; k++) {
    if (!spectral) {
      double* out = (double*)(w2 + 4 * g.fsc);  // n doubles fit in one 16-byte complex field
      k_flux_point<TS, true><<<nb, 256, 0, stream>>>(real, n, nin, k, out, ps, P, h_st->inv_tau);
      LAPS_CK(cudaGetLastError());
      LAPS_CK(cudaMemcpyAsync(host + k * n, out, n * sizeof(double), cudaMemcpyDeviceToHost, stream));
    } else {
      SRS* fr = (SRS*)(w2 + 4 * g.fsc);  // the flux field (state-type reals)
      k_flux_point<TS, false><<<nb, 256, 0, stream>>>(real, n, nin, k, fr, ps, P, h_st->inv_tau);
      LAPS_CK(cudaGetLastError());
      forward3d(fr, slot, 1);  // W2 field 0 as scratch
      double2* ref = (double2*)(w2 + 8 * g.fsc);
      k_spec_to_ref<TS><<<nb, 256, 0, stream>>>(slot, ref, g, 1);
      LAPS_CK(cudaGetLastError());
      LAPS_CK(cudaMemcpyAsync(host + 2 * k * nspec, ref, nspec * sizeof(double2), cudaMemcpyDeviceToHost, stream));
    }
    wait(tmo());
  }
}

// calc_rhs (mhdrhs.f90:174-279) alone: the fused passes over the whole spectrum with pass E
// storing fnl (with the expansion and explicit-diffusion terms, before rkt) in R; the state
// is left as it was.  Overwrites the RK register, so it belongs between steps.
template <class T, class TS> void Engine<T, TS>::calc_rhs(double* host) {
  if (!have_state) throw Error{LAPS_ESTATE, "no state uploaded"};
  if (P.variant == LAPS_VARIANT_3DI) throw Error{LAPS_EINVAL, "laps_calc_rhs serves the compressible variants"};
  const Geo& g = gfull;
  const bool was = dealiased;
  rhs_mode = true;
  force_full = true;
  try {
    LAPS_CK(cudaMemsetAsync(&st->halt, 0, sizeof(int), stream));
    enqueue_stage(0, false, true);
  } catch (...) {
    rhs_mode = force_full = false;
    dealiased = was;
    throw;
  }
  rhs_mode = force_full = false;
  dealiased = was;
  double2* ref = (double2*)B.W1;
  k_spec_to_ref<T><<<1024, 256, 0, stream>>>(B.R, ref, g, 8);
  LAPS_CK(cudaGetLastError());
  LAPS_CK(cudaMemcpyAsync(host, ref, (size_t)8 * g.nz * g.ny * g.nh * sizeof(double2), cudaMemcpyDeviceToHost, stream));
  wait(tmo());
}

// dealias (dealiasing.f90:70-113) applied to the state
template <class T, class TS> void Engine<T, TS>::dealias_state() {
  if (!have_state) throw Error{LAPS_ESTATE, "no state uploaded"};
  k_dealias_state<TS><<<1024, 256, 0, stream>>>(B.U, gfull, ktab_s(), P);
  LAPS_CK(cudaGetLastError());
  wait(tmo());
}

// ---------------------------------------------------------------------------- diagnostics
template <class T, class TS> void Engine<T, TS>::spectrum(int nshell, double* eu, double* eb) {
  if (!have_state) throw Error{LAPS_ESTATE, "no state uploaded"};
  if (nshell < 1 || nshell > 2048) throw Error{LAPS_EINVAL, "nshell must be in [1, 2048]"};
  const Geo& g = gfull;
  read_state();
  // velocity u = (rho u) / rho in real space, then its half spectrum in W2 fields 3..5
  inverse3d(B.U, 4);
  k_velocity<TS><<<1024, 256, 0, stream>>>((SRS*)B.W1, g.fsr);
  LAPS_CK(cudaGetLastError());
  CS* uh = W2s() + 3 * g.fsc;
  forward3d((const SRS*)B.W1 + g.fsr, uh, 3);
  const int nb = 304;
  const size_t need = (size_t)nb * 2 * nshell;
  if (spec_cap < need) {
    d_spec = dalloc<double>(need);
    spec_cap = need;
  }
  double lmax = std::fmax(p.Lx, p.Ly);
  if (p.nz > 1) lmax = std::fmax(lmax, p.Lz);
  const double dk = 2.0 * 3.141592653589793 / lmax;
  const int smem = SPEC_WARPS * 2 * nshell * (int)sizeof(double);
  set_smem(k_shell_spectrum<TS>, smem);
  k_shell_spectrum<TS><<<nb, SPEC_WARPS * 32, smem, stream>>>(uh, B.U + 4 * g.fsc, g.fsc, g, d_wx, d_wy, d_wz, 1.0 / dk,
                                                              nshell, d_spec);
  LAPS_CK(cudaGetLastError());
  std::vector<double> part(need);
  LAPS_CK(cudaMemcpyAsync(part.data(), d_spec, need * sizeof(double), cudaMemcpyDeviceToHost, stream));
  wait(tmo());
  for (int s = 0; s < nshell; s++) {
    double a = 0.0, b = 0.0;
    for (int k = 0; k < nb; k++) {
      a += part[(size_t)k * 2 * nshell + s];
      b += part[(size_t)k * 2 * nshell + nshell + s];
    }
    if (eu) eu[s] = a;
    if (eb) eb[s] = b;
  }
}

template <class T, class TS> void Engine<T, TS>::diagnostics(laps_diag* d) {
  if (!have_state) throw Error{LAPS_ESTATE, "no state uploaded"};
  const Geo& g = gfull;
  read_state();
  d->time = h_st->time;
  d->dt = h_st->dt;
  d->radius = h_st->radius;
  inverse3d(B.U, 8);  // real conserved T fields in W1
  int nb = npart;
  // pass 1: sums of f and f^2 for the 8 reported fields, the energies and u.B
  k_diag_sums<TS><<<nb, 256, 0, stream>>>((const SRS*)B.W1, g.fsr, P.gamma, P.variant == LAPS_VARIANT_3DI, d_part);
  LAPS_CK(cudaGetLastError());
  std::vector<double> part((size_t)nb * 32);
  LAPS_CK(cudaMemcpyAsync(part.data(), d_part, part.size() * sizeof(double), cudaMemcpyDeviceToHost, stream));
  wait(tmo());
  double s[32] = {0};
  for (int b = 0; b < nb; b++)
    for (int k = 0; k < 19; k++) s[k] += part[(size_t)b * 32 + k];
  double n = (double)g.fsr;
  double ave[8];
  for (int k = 0; k < 8; k++) {
    ave[k] = s[k] / n;
    d->uu_ave[k] = ave[k];
    d->uu_rms[k] = s[8 + k] / n - ave[k] * ave[k];
  }
  d->e_kin = 0.5 * s[16] / n;
  d->e_mag = 0.5 * s[17] / n;
  d->h_cross = s[18] / n;
  // pass 2: rho (u - <u>)^2
  k_diag_rhou2<TS><<<nb, 256, 0, stream>>>((const SRS*)B.W1, g.fsr, ave[1], ave[2], ave[3], d_part);
  LAPS_CK(cudaGetLastError());
  // spectral: max |ik.B| and <A.B>
  k_diag_spec<TS><<<nb, 256, 0, stream>>>(B.U, g, ktab_s(), P, ps, st, d_part + (size_t)nb * 8);
  LAPS_CK(cudaGetLastError());
  LAPS_CK(cudaMemcpyAsync(part.data(), d_part, part.size() * sizeof(double), cudaMemcpyDeviceToHost, stream));
  wait(tmo());
  double r2[3] = {0, 0, 0}, hm = 0, mx = 0;
  for (int b = 0; b < nb; b++) {
    for (int k = 0; k < 3; k++) r2[k] += part[(size_t)b * 8 + k];
    mx = std::fmax(mx, part[(size_t)nb * 8 + (size_t)b * 2 + 0]);
    hm += part[(size_t)nb * 8 + (size_t)b * 2 + 1];
  }
  for (int k = 0; k < 3; k++) d->rho_u2[k] = r2[k] / n;
  d->max_divB = mx;
  d->h_mag = hm;
  // real-space maxima of div B and div(rho u)/rho0 (the incompressible code's diagnostics)
  double mreal[2];
  for (int w = 0; w < 2; w++) {
    CS* spec = W2s() + (w2_fields(p) * WE / (long long)sizeof(CS) - 1) * g.fsc;
    k_spec_div<TS><<<1024, 256, 0, stream>>>(B.U, spec, g, ktab_s(), P, ps, st, w == 0 ? 4 : 1, w == 1);
    LAPS_CK(cudaGetLastError());
    inverse3d(spec, 1);
    k_max_abs<TS><<<nb, 256, 0, stream>>>((const SRS*)B.W1, g.fsr, d_part);
    LAPS_CK(cudaGetLastError());
    LAPS_CK(cudaMemcpyAsync(part.data(), d_part, (size_t)nb * sizeof(double), cudaMemcpyDeviceToHost, stream));
    wait(tmo());
    double m = 0;
    for (int b = 0; b < nb; b++) m = std::fmax(m, part[b]);
    mreal[w] = m;
  }
  d->max_divB_real = mreal[0];
  d->max_divV_real = mreal[1];
}

}  // namespace laps
