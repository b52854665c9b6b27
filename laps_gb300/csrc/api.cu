// C-ABI of the engine (declared in include/laps_gpu.h).  Every entry point converts
// exceptions into LAPS_E* codes; nothing C++ crosses the boundary.
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <thread>
#include <vector>
#include "engine_impl.cuh"

namespace laps {
EngineBase* make_engine_fp64(const laps_params& p);
EngineBase* make_engine_dd(const laps_params& p);
long long plan_bytes_fp64(const laps_params& p);
long long plan_bytes_dd(const laps_params& p);
EngineBase* make_engine_f32(const laps_params& p);
long long plan_bytes_f32(const laps_params& p);
EngineBase* make_engine_f32d(const laps_params& p);
long long plan_bytes_f32d(const laps_params& p);
}  // namespace laps

struct laps_ctx {
  laps::EngineBase* e = nullptr;
  std::string err;
};

static thread_local std::string g_create_err;

// used by entry points that have no context
void laps_set_create_error(const std::string& m) { g_create_err = m; }

static int fail(laps_ctx* c, int code, const std::string& m) {
  if (c) c->err = m;
  else g_create_err = m;
  return code;
}

template <class F> static int guarded(laps_ctx* c, F f) {
  if (!c || !c->e) return fail(c, LAPS_EINVAL, "null context");
  try {
    f();
    return LAPS_OK;
  } catch (const laps::Error& e) {
    return fail(c, e.code, e.msg);
  } catch (const std::bad_alloc&) {
    return fail(c, LAPS_ENOMEM, "host allocation failed");
  } catch (...) {
    return fail(c, LAPS_ECUDA, "unexpected error");
  }
}

extern "C" {

int laps_params_default(laps_params* p) {
  if (!p) return LAPS_EINVAL;
  std::memset(p, 0, sizeof(*p));
  const double pi = 3.141592653589793;
  p->variant = LAPS_VARIANT_3DC;
  p->precision = LAPS_PREC_FP64;
  p->nx = 128; p->ny = 128; p->nz = 64;  // mhdinit.f90:5
  p->Lx = p->Ly = p->Lz = 2 * pi;
  p->adiabatic_index = 5.0 / 3.0;      // mhdinit.f90:21
  p->dealias_option = 2;               // dealiasing.f90:11
  p->afx = p->afy = p->afz = 0.495;    // dealiasing.f90:12
  p->cfl = 0.5;                        // mhd.f90:21
  p->radius0 = 30.0;                   // AEBmod.f90:12
  p->rho0 = 1.0;                       // src_incompressible/mhdinit.f90:15
  p->dstep_calcdt = 20;                // src_compressible/2D/mhd.f90:20 (2-D only)
  p->timeout_ms = 600000;
  return LAPS_OK;
}

static bool size_ok(int n, int lo) { return n >= lo && n <= 1024 && (n & (n - 1)) == 0; }

int laps_create(const laps_params* p, laps_ctx** out) {
  if (!p || !out) return fail(nullptr, LAPS_EINVAL, "null argument");
  *out = nullptr;
  if (p->variant != LAPS_VARIANT_3DC && p->variant != LAPS_VARIANT_3DI && p->variant != LAPS_VARIANT_2DC)
    return fail(nullptr, LAPS_EINVAL, "variant must be LAPS_VARIANT_3DC, LAPS_VARIANT_3DI or LAPS_VARIANT_2DC");
  if (p->precision < LAPS_PREC_FP64 || p->precision > LAPS_PREC_FP32_F64)
    return fail(nullptr, LAPS_EINVAL, "precision must be LAPS_PREC_FP64, LAPS_PREC_DD, LAPS_PREC_FP32 or LAPS_PREC_FP32_F64");
  if (p->variant == LAPS_VARIANT_2DC) {
    if (!size_ok(p->nx, 16) || !size_ok(p->ny, 8) || p->nz != 1)
      return fail(nullptr, LAPS_EINVAL, "2-D: nx a power of two in [16,1024], ny in [8,1024], nz = 1");
    if (p->dstep_calcdt < 1) return fail(nullptr, LAPS_EINVAL, "dstep_calcdt must be >= 1");
    if (p->if_AEB && p->if_z_radial && p->if_corotating)
      return fail(nullptr, LAPS_EINVAL, "if_z_radial and if_corotating cannot both be set (src_compressible/2D/mhd.f90:59-68)");
  } else if (!size_ok(p->nx, 16) || !size_ok(p->ny, 8) || !size_ok(p->nz, 8) || p->nx > 512 || p->ny > 512 || p->nz > 512) {
    return fail(nullptr, LAPS_EINVAL, "3-D: nx a power of two in [16,512], ny and nz in [8,512]");
  }
  if (p->variant == LAPS_VARIANT_3DI && !(p->rho0 > 0)) return fail(nullptr, LAPS_EINVAL, "rho0 must be positive");
  if (!(p->Lx > 0 && p->Ly > 0 && p->Lz > 0)) return fail(nullptr, LAPS_EINVAL, "box lengths must be positive");
  if (!(p->adiabatic_index != 1.0) || !(p->cfl > 0)) return fail(nullptr, LAPS_EINVAL, "adiabatic_index must differ from 1 and cfl be positive");
  if (p->if_AEB && !(p->radius0 > 0)) return fail(nullptr, LAPS_EINVAL, "radius0 must be positive");
  long long need = p->precision == LAPS_PREC_FP64 ? laps::plan_bytes_fp64(*p)
                   : p->precision == LAPS_PREC_DD ? laps::plan_bytes_dd(*p)
                   : p->precision == LAPS_PREC_FP32 ? laps::plan_bytes_f32(*p)
                                                    : laps::plan_bytes_f32d(*p);
  if (p->mem_cap_bytes > 0 && need > p->mem_cap_bytes)
    return fail(nullptr, LAPS_ENOMEM, "device memory needed (" + std::to_string(need) + " bytes) exceeds mem_cap_bytes");
  laps_ctx* c = new (std::nothrow) laps_ctx;
  if (!c) return fail(nullptr, LAPS_ENOMEM, "host allocation failed");
  try {
    c->e = p->precision == LAPS_PREC_FP64 ? laps::make_engine_fp64(*p)
           : p->precision == LAPS_PREC_DD ? laps::make_engine_dd(*p)
           : p->precision == LAPS_PREC_FP32 ? laps::make_engine_f32(*p)
                                            : laps::make_engine_f32d(*p);
  } catch (const laps::Error& e) {
    delete c;
    return fail(nullptr, e.code, e.msg);
  } catch (...) {
    delete c;
    return fail(nullptr, LAPS_ECUDA, "engine construction failed");
  }
  *out = c;
  return LAPS_OK;
}

void laps_destroy(laps_ctx* c) {
  if (!c) return;
  delete c->e;
  delete c;
}

int laps_upload_state(laps_ctx* c, const double* uu, int layout) {
  if (!uu || (layout != LAPS_LAYOUT_PRIMITIVE && layout != LAPS_LAYOUT_CONSERVED)) return fail(c, LAPS_EINVAL, "bad state pointer or layout");
  return guarded(c, [&] { c->e->upload(uu, layout); });
}
int laps_ic_default(laps_ic* ic) {
  if (!ic) return LAPS_EINVAL;
  std::memset(ic, 0, sizeof(*ic));
  ic->T0 = 1.0; ic->rho0 = 1.0;  // mhdinit.f90:13
  ic->B0 = 1.0; ic->a0 = 0.05;   // mhdinit.f90:14
  ic->in_out_ratio = 1.0;        // mhdinit.f90:48-49
  ic->nmodex = ic->nmodey = ic->nmodez = 16;  // mhdinit.f90:50
  ic->jet_width = 1.0; ic->Vjet = 0.3; ic->wave_number_jet = 1;  // mhdinit.f90:52-53
  return LAPS_OK;
}
long long laps_ic_nphases(const laps_ic* ic) {
  if (!ic) return 0;
  const long long mx = ic->nmodex, my = ic->nmodey, mz = ic->nmodez;
  if (ic->ipert == 6) return 2 * mx * (2 * my + 1) * (2 * mz + 1);
  if (ic->ipert == 7) return 3 * (2 * mx + 1) * (2 * my + 1) * (2 * mz + 1);
  return 0;
}
int laps_init_fields(laps_ctx* c, const laps_ic* ic, const double* phases, long long nphases) {
  if (!c) return LAPS_EINVAL;
  if (!ic) return fail(c, LAPS_EINVAL, "null initial-condition parameters");
  const laps_params& q = c->e->params();
  if (q.variant == LAPS_VARIANT_2DC) return fail(c, LAPS_EINVAL, "initial conditions are generated for the 3-D variants only");
  if (ic->ifield < 0 || ic->ifield > 5 || (ic->ifield == 5 && q.variant != LAPS_VARIANT_3DC))
    return fail(c, LAPS_EINVAL, "ifield must be 0-4 (0-5 for the 3-D compressible variant)");
  if (ic->ipert != 0 && ic->ipert != 1 && ic->ipert != 6 && ic->ipert != 7 && ic->ipert != 8)
    return fail(c, LAPS_EINVAL, "ipert must be 0, 1, 6, 7 or 8 (2-5 are not built)");
  if ((ic->ifield == 1 || ic->ifield == 4) && ic->a0 == 0.0) return fail(c, LAPS_EINVAL, "a0 = 0");
  if (ic->ifield == 2 && ic->shear_width == 0.0) return fail(c, LAPS_EINVAL, "shear_width = 0");
  if (ic->ifield == 1 && ic->T0 == 0.0) return fail(c, LAPS_EINVAL, "T0 = 0");
  if (ic->ipert == 8 && (ic->R1_SB == 0.0 || ic->H_SB == 0.0 || ic->Rd_SB == 0.0))
    return fail(c, LAPS_EINVAL, "switchback widths R1_SB, H_SB, Rd_SB must be non-zero");
  const long long need = laps_ic_nphases(ic);
  if (need > 0) {
    if (ic->nmodex < 1 || ic->nmodey < 0 || ic->nmodez < 0) return fail(c, LAPS_EINVAL, "nmodex >= 1, nmodey, nmodez >= 0");
    if (2 * ic->nmodex >= q.nx || 2 * ic->nmodey >= q.ny || 2 * ic->nmodez >= q.nz)
      return fail(c, LAPS_EINVAL, "random-phase modes need nmodex < nx/2, nmodey < ny/2, nmodez < nz/2");
    if (!phases || nphases != need) return fail(c, LAPS_EINVAL, "phases: laps_ic_nphases(ic) values expected");
    if (ic->ipert == 7 && ic->bx0 == 0.0 && ic->by0 == 0.0 && ic->bz0 == 0.0)
      return fail(c, LAPS_EINVAL, "ipert 7 needs a non-zero background field (bx0, by0, bz0)");
  }
  return guarded(c, [&] { c->e->init_fields(*ic, phases); });
}
int laps_angle_statistics(laps_ctx* c, int axis, double* out) {
  if (!c) return LAPS_EINVAL;
  if (axis < 0 || axis > 2 || !out) return fail(c, LAPS_EINVAL, "axis must be 0, 1 or 2 and out non-null");
  return guarded(c, [&] { c->e->angle_statistics(axis, out); });
}
int laps_set_time(laps_ctx* c, double t) { return guarded(c, [&] { c->e->set_time(t); }); }
int laps_vardt(laps_ctx* c, double* dt) {
  return guarded(c, [&] {
    double d = c->e->vardt();
    if (dt) *dt = d;
  });
}
int laps_step(laps_ctx* c, int n, double* time, double* dt, int* status) {
  if (n < 0) return fail(c, LAPS_EINVAL, "nsteps < 0");
  return guarded(c, [&] { c->e->step(n, time, dt, status); });
}
int laps_step_profiled(laps_ctx* c, int n, double* pass_ms, double* total_ms, int* status) {
  if (n < 1 || !pass_ms || !total_ms) return fail(c, LAPS_EINVAL, "bad arguments");
  return guarded(c, [&] { c->e->step_profiled(n, pass_ms, total_ms, status); });
}
int laps_rk_stage(laps_ctx* c, int irk) { return guarded(c, [&] { c->e->rk_stage(irk); }); }
int laps_download_state(laps_ctx* c, double* uu, double* prim) { return guarded(c, [&] { c->e->download(uu, prim); }); }
int laps_download_spectral(laps_ctx* c, double* uf) {
  if (!uf) return fail(c, LAPS_EINVAL, "null array");
  return guarded(c, [&] { c->e->download_spectral(uf); });
}
int laps_upload_spectral(laps_ctx* c, const double* uf) {
  if (!uf) return fail(c, LAPS_EINVAL, "null array");
  return guarded(c, [&] { c->e->upload_spectral(uf); });
}
int laps_diagnostics(laps_ctx* c, laps_diag* d) {
  if (!d) return fail(c, LAPS_EINVAL, "null diag");
  return guarded(c, [&] { c->e->diagnostics(d); });
}
int laps_spectrum(laps_ctx* c, int nshell, double* e_u, double* e_b) {
  if (!e_u && !e_b) return fail(c, LAPS_EINVAL, "null spectrum arrays");
  return guarded(c, [&] { c->e->spectrum(nshell, e_u, e_b); });
}
int laps_calc_flux(laps_ctx* c, double* flux) {
  if (!flux) return fail(c, LAPS_EINVAL, "null output");
  return guarded(c, [&] { c->e->calc_flux(flux, 0); });
}
int laps_transform_flux(laps_ctx* c, double* flux_fourier) {
  if (!flux_fourier) return fail(c, LAPS_EINVAL, "null output");
  return guarded(c, [&] { c->e->calc_flux(flux_fourier, 1); });
}
int laps_calc_rhs(laps_ctx* c, double* fnl) {
  if (!fnl) return fail(c, LAPS_EINVAL, "null output");
  return guarded(c, [&] { c->e->calc_rhs(fnl); });
}
int laps_dealias(laps_ctx* c) { return guarded(c, [&] { c->e->dealias_state(); }); }
int laps_set_schedule(laps_ctx* c, int bits) { return guarded(c, [&] { c->e->set_schedule(bits); }); }
int laps_get_schedule(laps_ctx* c, int* bits) {
  if (!bits) return fail(c, LAPS_EINVAL, "null output pointer");
  return guarded(c, [&] { *bits = c->e->schedule(); });
}
int laps_state_real_device(laps_ctx* c, double* uu_dev) {
  if (!uu_dev) return fail(c, LAPS_EINVAL, "null buffer");
  return guarded(c, [&] { c->e->state_real_device(uu_dev); });
}
int laps_add_spectral_device(laps_ctx* c, const double* duf_dev, double scale) {
  if (!duf_dev) return fail(c, LAPS_EINVAL, "null buffer");
  return guarded(c, [&] { c->e->add_spectral_device(duf_dev, scale); });
}
int laps_transform_uu_k2r(laps_ctx* c, double* uu) {
  if (!uu) return fail(c, LAPS_EINVAL, "null output");
  return guarded(c, [&] { c->e->download(uu, nullptr); });
}
int laps_update_prim(laps_ctx* c, double* uu_prim) {
  if (!uu_prim) return fail(c, LAPS_EINVAL, "null output");
  return guarded(c, [&] { c->e->download(nullptr, uu_prim); });
}
int laps_wait(laps_ctx* c, int timeout_ms) { return guarded(c, [&] { c->e->wait(timeout_ms); }); }
int laps_get_time(laps_ctx* c, double* t, double* dt) { return guarded(c, [&] { c->e->get_time(t, dt); }); }
int laps_get_info(laps_ctx* c, laps_info* i) {
  if (!i) return fail(c, LAPS_EINVAL, "null info");
  return guarded(c, [&] { c->e->info(i); });
}
const char* laps_last_error(laps_ctx* c) { return c ? c->err.c_str() : g_create_err.c_str(); }

}  // extern "C"

// ---------------------------------------------------------------------------- ensembles
// A batch owns n member contexts on one device, each with its own stream.  Its step replays
// one CUDA graph per step: a fork from the batch's stream to every member's stream, each
// member's step kernels, and a join back.  Members therefore run concurrently (a 128^2 member
// alone fills a few SMs) and keep their own dt, cadence and status.
using laps::Error;  // LAPS_CK throws laps::Error

struct laps_batch {
  std::vector<laps_ctx*> m;
  cudaStream_t origin = nullptr;
  cudaGraphExec_t graph = nullptr;
  long long sched_changes = 0;  // members' schedule changes when the graph was captured
  cudaEvent_t ev_fork = nullptr, ev_done = nullptr;
  std::vector<cudaEvent_t> ev_join;
  int dev = 0;
  int timeout_ms = 600000;
  std::string err;
};

static void batch_free(laps_batch* b) {
  if (!b) return;
  if (b->graph) cudaGraphExecDestroy(b->graph);
  for (cudaEvent_t e : b->ev_join) cudaEventDestroy(e);
  if (b->ev_fork) cudaEventDestroy(b->ev_fork);
  if (b->ev_done) cudaEventDestroy(b->ev_done);
  if (b->origin) cudaStreamDestroy(b->origin);
  for (laps_ctx* c : b->m) laps_destroy(c);
  delete b;
}

// bounded wait for everything enqueued on `s` (the same rule as laps_wait)
static void wait_stream(cudaStream_t s, cudaEvent_t ev, int timeout_ms) {
  LAPS_CK(cudaEventRecord(ev, s));
  auto t0 = std::chrono::steady_clock::now();
  for (;;) {
    cudaError_t e = cudaEventQuery(ev);
    if (e == cudaSuccess) return;
    if (e != cudaErrorNotReady) throw laps::Error{LAPS_ECUDA, std::string("device error: ") + cudaGetErrorString(e)};
    auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::steady_clock::now() - t0).count();
    if (timeout_ms > 0 && ms > timeout_ms) throw laps::Error{LAPS_ETIMEDOUT, "device work did not finish within the timeout"};
    std::this_thread::sleep_for(std::chrono::microseconds(50));
  }
}

extern "C" {

int laps_batch_create(const laps_params* members, int n, laps_batch** out) {
  if (!out) return fail(nullptr, LAPS_EINVAL, "null output pointer");
  *out = nullptr;
  if (!members || n < 1 || n > 4096) return fail(nullptr, LAPS_EINVAL, "members must hold 1..4096 parameter sets");
  for (int i = 1; i < n; i++)
    if (members[i].device != members[0].device) return fail(nullptr, LAPS_EINVAL, "all members must use one device");
  laps_batch* b = new (std::nothrow) laps_batch;
  if (!b) return fail(nullptr, LAPS_ENOMEM, "host allocation failed");
  b->dev = members[0].device;
  for (int i = 0; i < n; i++) {
    laps_ctx* c = nullptr;
    int rc = laps_create(&members[i], &c);
    if (rc != LAPS_OK) {
      std::string m = "member " + std::to_string(i) + ": " + g_create_err;
      batch_free(b);
      return fail(nullptr, rc, m);
    }
    b->m.push_back(c);
    if (members[i].timeout_ms > b->timeout_ms) b->timeout_ms = members[i].timeout_ms;
  }
  try {
    LAPS_CK(cudaSetDevice(b->dev));
    LAPS_CK(cudaStreamCreateWithFlags(&b->origin, cudaStreamNonBlocking));
    LAPS_CK(cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming));
    LAPS_CK(cudaEventCreateWithFlags(&b->ev_done, cudaEventDisableTiming));
    b->ev_join.resize(n, nullptr);
    for (int i = 0; i < n; i++) LAPS_CK(cudaEventCreateWithFlags(&b->ev_join[i], cudaEventDisableTiming));
  } catch (const laps::Error& e) {
    batch_free(b);
    return fail(nullptr, e.code, e.msg);
  }
  *out = b;
  return LAPS_OK;
}

void laps_batch_destroy(laps_batch* b) { batch_free(b); }

int laps_batch_size(laps_batch* b) { return b ? (int)b->m.size() : 0; }

int laps_batch_member(laps_batch* b, int i, laps_ctx** ctx) {
  if (!b || !ctx) return fail(nullptr, LAPS_EINVAL, "null batch or output pointer");
  if (i < 0 || i >= (int)b->m.size()) {
    b->err = "member index out of range";
    return LAPS_EINVAL;
  }
  *ctx = b->m[i];
  return LAPS_OK;
}

int laps_batch_step(laps_batch* b, int nsteps, double* time, double* dt, int* status) {
  if (!b) return fail(nullptr, LAPS_EINVAL, "null batch");
  if (nsteps < 0) {
    b->err = "nsteps must be >= 0";
    return LAPS_EINVAL;
  }
  const int n = (int)b->m.size();
  for (int i = 0; i < n; i++)
    if (!b->m[i]->e->has_state()) {
      b->err = "member " + std::to_string(i) + ": no state uploaded";
      return LAPS_ESTATE;
    }
  try {
    LAPS_CK(cudaSetDevice(b->dev));
    bool first = false;
    for (int i = 0; i < n; i++) {
      b->m[i]->e->reset_flags();
      first = first || b->m[i]->e->needs_first_step();
    }
    int done = 0;
    if (nsteps > 0 && first) {  // unpruned first steps, each member on its own stream
      for (int i = 0; i < n; i++) b->m[i]->e->enqueue_one_step();
      done = 1;
    }
    if (done < nsteps) {
      for (int i = 0; i < n; i++) {  // the graph starts after every member's pending work
        LAPS_CK(cudaEventRecord(b->ev_join[i], b->m[i]->e->get_stream()));
        LAPS_CK(cudaStreamWaitEvent(b->origin, b->ev_join[i], 0));
      }
      long long changes = 0;  // a member's schedule changed since the capture: capture again
      for (int i = 0; i < n; i++) changes += b->m[i]->e->schedule_changes();
      if (b->graph && changes != b->sched_changes) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
      }
      b->sched_changes = changes;
      if (!b->graph) {
        cudaGraph_t gr;
        LAPS_CK(cudaStreamBeginCapture(b->origin, cudaStreamCaptureModeThreadLocal));
        LAPS_CK(cudaEventRecord(b->ev_fork, b->origin));
        for (int i = 0; i < n; i++) {
          cudaStream_t s = b->m[i]->e->get_stream();
          LAPS_CK(cudaStreamWaitEvent(s, b->ev_fork, 0));
          b->m[i]->e->enqueue_one_step();
          LAPS_CK(cudaEventRecord(b->ev_join[i], s));
          LAPS_CK(cudaStreamWaitEvent(b->origin, b->ev_join[i], 0));
        }
        LAPS_CK(cudaStreamEndCapture(b->origin, &gr));
        cudaError_t e = cudaGraphInstantiate(&b->graph, gr, 0);
        cudaGraphDestroy(gr);
        LAPS_CK(e);
      }
      for (; done < nsteps; done++) LAPS_CK(cudaGraphLaunch(b->graph, b->origin));
      LAPS_CK(cudaEventRecord(b->ev_done, b->origin));
      for (int i = 0; i < n; i++) LAPS_CK(cudaStreamWaitEvent(b->m[i]->e->get_stream(), b->ev_done, 0));
    }
    wait_stream(b->origin, b->ev_done, b->timeout_ms);
    for (int i = 0; i < n; i++)
      b->m[i]->e->host_state(time ? time + i : nullptr, dt ? dt + i : nullptr, status ? status + i : nullptr);
  } catch (const laps::Error& e) {
    b->err = e.msg;
    return e.code;
  } catch (...) {
    b->err = "unexpected error";
    return LAPS_ECUDA;
  }
  return LAPS_OK;
}

const char* laps_batch_last_error(laps_batch* b) { return b ? b->err.c_str() : g_create_err.c_str(); }

}  // extern "C"

// ---------------------------------------------------------------------------- output files
// The reference's outNNN.dat (mhdoutput.f90:72-131, restart.f90:17-63): a Fortran unformatted
// sequential record holding the time as a 4-byte real (4-byte length markers: 12 bytes), then
// uu(nx,ny,nz,8) as 8-byte reals in Fortran order from byte 12 (the MPI-IO view's displacement;
// the reference is built with -r8).  Primitive output replaces rho u by u and, in the
// compressible codes, e by p; the incompressible state already holds p.

namespace {

struct PinnedPair {  // two page-locked bounce buffers for overlapped copies and file I/O
  double* buf[2] = {nullptr, nullptr};
  cudaEvent_t ev[2] = {nullptr, nullptr};
  explicit PinnedPair(size_t n) {
    for (int i = 0; i < 2; i++) {
      LAPS_CK(cudaMallocHost(&buf[i], n * sizeof(double)));
      LAPS_CK(cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming));
    }
  }
  ~PinnedPair() {
    for (int i = 0; i < 2; i++) {
      if (buf[i]) cudaFreeHost(buf[i]);
      if (ev[i]) cudaEventDestroy(ev[i]);
    }
  }
};

void wait_event(cudaEvent_t ev, int timeout_ms) {
  auto t0 = std::chrono::steady_clock::now();
  for (;;) {
    cudaError_t e = cudaEventQuery(ev);
    if (e == cudaSuccess) return;
    if (e != cudaErrorNotReady) throw laps::Error{LAPS_ECUDA, std::string("device error: ") + cudaGetErrorString(e)};
    auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::steady_clock::now() - t0).count();
    if (timeout_ms > 0 && ms > timeout_ms) throw laps::Error{LAPS_ETIMEDOUT, "device work did not finish within the timeout"};
    std::this_thread::sleep_for(std::chrono::microseconds(50));
  }
}

struct File {
  FILE* f = nullptr;
  File(const char* path, const char* mode) : f(std::fopen(path, mode)) {}
  ~File() {
    if (f) std::fclose(f);
  }
};

constexpr size_t kChunk = size_t(1) << 22;  // doubles per bounce buffer (32 MiB)

}  // namespace

extern "C" {

int laps_write_output(laps_ctx* c, const char* path, int layout) {
  if (!path) return fail(c, LAPS_EINVAL, "null path");
  if (layout != LAPS_LAYOUT_PRIMITIVE && layout != LAPS_LAYOUT_CONSERVED) return fail(c, LAPS_EINVAL, "bad layout");
  return guarded(c, [&] {
    laps::EngineBase* e = c->e;
    double t = 0.0, dt = 0.0;
    e->get_time(&t, &dt);
    const double* dev = e->stage_real_state();
    const long long n = e->grid_points();
    cudaStream_t s = e->get_stream();
    File out(path, "wb");
    if (!out.f) throw laps::Error{LAPS_EINVAL, std::string("cannot open ") + path + " for writing"};
    const int32_t mark = 4;
    const float t4 = (float)t;
    bool ok = std::fwrite(&mark, 4, 1, out.f) == 1 && std::fwrite(&t4, 4, 1, out.f) == 1 && std::fwrite(&mark, 4, 1, out.f) == 1;
    // field f of the file: conserved slot f, or u (prim 0..2) for slots 1..3 and p (prim 3)
    // for slot 7 of the compressible codes
    const bool prim = layout == LAPS_LAYOUT_PRIMITIVE;
    const bool incomp = e->variant() == LAPS_VARIANT_3DI;
    auto src = [&](int f) -> const double* {
      if (prim && f >= 1 && f <= 3) return dev + (8 + f - 1) * n;
      if (prim && f == 7 && !incomp) return dev + 11 * n;
      return dev + (long long)f * n;
    };
    PinnedPair pp((size_t)std::min<long long>(n * 8, (long long)kChunk));
    // chunks over the 8 fields; the copy of chunk i+1 runs while chunk i is written
    struct Piece { const double* p; size_t cnt; };
    std::vector<Piece> pieces;
    for (int f = 0; f < 8; f++)
      for (long long o = 0; o < n; o += (long long)kChunk) pieces.push_back({src(f) + o, (size_t)std::min<long long>(kChunk, n - o)});
    auto issue = [&](size_t i) {
      const int b = (int)(i & 1);
      LAPS_CK(cudaMemcpyAsync(pp.buf[b], pieces[i].p, pieces[i].cnt * sizeof(double), cudaMemcpyDeviceToHost, s));
      LAPS_CK(cudaEventRecord(pp.ev[b], s));
    };
    if (!pieces.empty()) issue(0);
    for (size_t i = 0; i < pieces.size(); i++) {
      const int b = (int)(i & 1);
      wait_event(pp.ev[b], 600000);
      if (i + 1 < pieces.size()) issue(i + 1);
      ok = ok && std::fwrite(pp.buf[b], sizeof(double), pieces[i].cnt, out.f) == pieces[i].cnt;
    }
    if (!ok) throw laps::Error{LAPS_EINVAL, std::string("write failed: ") + path};
  });
}

int laps_read_restart(laps_ctx* c, const char* path, double* time) {
  if (!path) return fail(c, LAPS_EINVAL, "null path");
  return guarded(c, [&] {
    laps::EngineBase* e = c->e;
    const long long n = e->grid_points();
    File in(path, "rb");
    if (!in.f) throw laps::Error{LAPS_EINVAL, std::string("cannot open ") + path};
    int32_t m0 = 0, m1 = 0;
    float t4 = 0.f;
    if (std::fread(&m0, 4, 1, in.f) != 1 || std::fread(&t4, 4, 1, in.f) != 1 || std::fread(&m1, 4, 1, in.f) != 1 || m0 != 4 || m1 != 4)
      throw laps::Error{LAPS_EINVAL, std::string("not an output file (bad time record): ") + path};
    std::vector<double> uu((size_t)n * 8);
    if (std::fread(uu.data(), sizeof(double), uu.size(), in.f) != uu.size())
      throw laps::Error{LAPS_EINVAL, std::string("output file too short for this grid: ") + path};
    e->upload(uu.data(), LAPS_LAYOUT_PRIMITIVE);
    const double t = (double)t4;  // the restart time goes through a 4-byte real
    e->set_time(t);
    if (time) *time = t;
  });
}

}  // extern "C"
