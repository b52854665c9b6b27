#!/usr/bin/env python3
"""Throughput of the LAPS RHS + RK3 step on GB300: grid-point-steps per second.

Workload: the 3-D compressible Hall-MHD run with the expanding box at 256^3 (d_i = 0.05,
Ur0/R0 = 0.01, eta = nu = 5e-4, 2/3 mask, cfl 0.4, random-phase 1 <= |k| <= 8 spectrum with
rms 0.5, seed 1), seeded synthetic initial condition.  A "step" is one full time step
(CFL, three RK stages, radius update) of the whole grid.

Our arm (default --precision fp32_f64): FP32 transforms and nonlinear products with the
state, RK accumulation, CFL reduction and diagnostics in IEEE FP64 - the FP32-FFT option the
target names - through the C-ABI, with its error against the FP64 engine stated over the
workload's 500 steps (`error_vs_fp64`: per-field relative L2, invariants, time and the E(k)
shell spectra of every shell up to k_max/2).  The other modes run beside it on the same
workload (`plain`: "fp32" with a float-float state, "dd" the float-float engine that matches
FP64 to 1e-10, "fp64" native binary64), each with its own roofline and end-to-end figure; the
FP64 line also carries `fp64_roofline` (its transform flops against the FP64 pipe).
`value` is device-timed with CUDA events on the engine's stream, state resident in HBM;
`e2e` is the same metric through the C-ABI with host buffers (pinned upload of the primitive
initial state, one laps_step call per step returning time/dt/status to the host, download of
the final state).  `cufft_yardstick` times cuFFT's unfused transforms of the same fields
beside the hand-written passes (outside the timed region).

--impl reference: the reference's CPU algorithm on the machine's host cores - the C++/OpenMP
restatement with its own FFT (oracle/laps3d_omp.cpp; the reference itself needs Fortran, MPI
and FFTW, which the box does not have) - timed over the same --warmup / --steps of the same
workload; `cpu_baseline` in our arm is the same code on a 1 + 5 step sample.

For N > 1 (torchrun) every rank advances its own independent replica ("replicas only":
one run does not shard); value = all ranks' grid-point-steps / the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "grid-point-steps/s vs plain FP64 at stated spectrum error; FFT HBM GB/s % peak"
N_GRID = 256
WORKLOAD = "3D compressible Hall-MHD + expanding box, 256^3"
CFG2 = dict(if_resis=1, resistivity=5e-4, if_visc=1, viscosity=5e-4, dealias_option=1, cfl=0.4,
            if_Hall=1, ion_inertial_length=0.05, if_AEB=1, radius0=30.0, Ur0=0.3)
CFG3 = dict(if_resis=1, resistivity=2e-4, if_visc=1, viscosity=2e-4, dealias_option=1, cfl=0.4, rho0=1.0)
SHAPE = None  # (nx, ny, nz) of a reduced profiling case
# workloads of the single-run arm: grid, variant, namelist values, description
WORKLOADS = {
    "c3d256": dict(grid=256, variant=0, kw=CFG2, label="3D compressible Hall-MHD + expanding box",
                   data="synthetic (seeded random-phase spectrum, 1<=|k|<=8, rms 0.5, seed 1)",
                   desc={"variant": "3DC", "hall": 0.05, "expanding_box": "Ur0/R0=0.01", "dealias": "2/3 sphere",
                         "cfl": 0.4}),
    "c3di512": dict(grid=512, variant=1, kw=CFG3, label="3D incompressible MHD",
                    data="synthetic (Taylor-Green-like u, b plus random-phase 1<=|k|<=6, |k|^-5/6, rms 1, seed 2)",
                    desc={"variant": "3DI", "eta_nu": 2e-4, "dealias": "2/3 sphere", "cfl": 0.4}),
}
WL = WORKLOADS["c3d256"]
# --precision: (C-ABI mode, dtype text, state bytes per complex, work-buffer bytes per complex)
PRECISIONS = {
    "dd": (1, "f32x2 (float-float)", 16, 16),
    "fp64": (0, "f64", 16, 16),
    "fp32": (2, "f32 transforms and products, f32x2 state / RK / CFL / diagnostics", 16, 8),
    "fp32_f64": (3, "f32 transforms and products, f64 state / RK / CFL / diagnostics", 16, 8),
}
PASS_NAMES = ["A_inv_z", "B_inv_y", "C_x_flux", "D_fwd_y", "E_fwd_z_rk", "bookkeeping"]


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def barrier_max(value: float, ws: int):
    if ws == 1:
        return value
    import torch
    import torch.distributed as dist

    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def initial_state(n=None):
    from laps_gb300.ic import taylor_green_ic, turbulence_ic

    n = n or (SHAPE if SHAPE else N_GRID)
    if WL["variant"] == 1:
        return taylor_green_ic(n, seed=2, kmin=1, kmax=6, alpha=-5.0 / 6.0, rms=1.0)
    return turbulence_ic(n, kmin=1, kmax=8, alpha=-1.0, rms_u=0.5, rms_b=0.5, seed=1)


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, dev):
        self.dev = dev
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.p = None
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.p is not None:
            self.p.terminate()
            try:
                self.out, _ = self.p.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()
                self.out, _ = self.p.communicate()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (self.out or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    try:
        d = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# algorithmic HBM bytes of one launch of each pass: compulsory reads + writes of the dataflow
# implemented.  eS / eT are the bytes of one complex element of the state (U, R) and of the work
# buffers (W1, W2); kx columns are moved in tiles of 8.  Steady-state stages: pruned to the
# kept modes, continuity taken from the momentum spectrum (mass=True), so pass C transforms 13
# flux fields (12 without the expansion term) and pass D writes 13 (15 without mass).
def pass_bytes(n, kx_keep, nky, nkz, hall=True, aeb=True, eS=16, eT=16, mass=True):
    kxp8 = int(math.ceil(kx_keep / 8.0) * 8)
    col_A = kxp8 * nky            # columns of pass A / E
    col_B = kxp8 * n              # columns of pass B / D (one per z plane)
    na = 10 if hall else 8        # pass A / B outputs (state + current components)
    nin = 8 + (3 if hall else 0)  # pass C inputs
    nfl = (13 if mass else 16) - (0 if aeb else 1)
    nd = 13 if mass else 15
    A = col_A * (8 * nkz * eS + na * n * eT)
    B = col_B * (na * nky * eT + nin * n * eT)
    C = n * n * kx_keep * (nin + nfl) * eT
    D = col_B * (nfl * n * eT + nd * nky * eT)
    E = col_A * (nd * n * eT + 8 * nkz * 2 * (eS + eT))  # U (state type) and R (work type) read and written
    return {"A_inv_z": A, "B_inv_y": B, "C_x_flux": C, "D_fwd_y": D, "E_fwd_z_rk": E}


# the same for one 2-D compressible member (nz = 1: no pass A; pass B reads the 8 state fields
# itself and writes 11 (state + current); pass E is elementwise over the kept (kx, ky) modes,
# the continuity update included); Hall on, expanding box off, continuity from the momentum
def pass_bytes_2d(n, kx_keep, nky, eS=16, eT=16):
    kxp8 = int(math.ceil(kx_keep / 8.0) * 8)
    na, nfl, nd = 11, 12, 13
    B = kxp8 * (8 * nky * eS + na * n * eT)
    C = n * kx_keep * (na + nfl) * eT
    D = kxp8 * (nfl * n * eT + nd * nky * eT)
    E = kxp8 * nky * (nd * eT + 8 * 2 * (eS + eT))
    return {"A_inv_z": 0, "B_inv_y": B, "C_x_flux": C, "D_fwd_y": D, "E_fwd_z_rk": E}


# the same for the incompressible step: A reads 7 state fields and writes 12 (u, B, J, grad
# terms), B 12 -> 19, C 19 -> 6 (pressure flux, E), D 6 -> 8, E reads 8 and updates 8 state
# fields (U and R read and written on kept kz)
def pass_bytes_3di(n, kx_keep, nky, nkz, eS=16, eT=16):
    kxp8 = int(math.ceil(kx_keep / 8.0) * 8)
    col_A, col_B = kxp8 * nky, kxp8 * n
    A = col_A * (7 * nkz * eS + 12 * n * eT)
    B = col_B * (12 * nky + 19 * n) * eT
    C = n * n * kx_keep * 25 * eT
    D = col_B * (6 * n + 8 * nky) * eT
    E = col_A * (8 * n * eT + 8 * nkz * 2 * (eS + eT))
    return {"A_inv_z": A, "B_inv_y": B, "C_x_flux": C, "D_fwd_y": D, "E_fwd_z_rk": E}


def cpu_sample(steps, warmup, n=None):
    """The reference's step restated for the host cores: the C++/OpenMP restatement
    (oracle/laps3d_omp.cpp, its own FFT, FP64, every host thread) - warmup + timed steps of
    the full grid.  Falls back to the numpy restatement where g++ / OpenMP cannot build it.
    Returns (grid-point-steps/s, threads, sample text, kind)."""
    n = n or N_GRID
    prim = initial_state(n)
    try:
        from oracle import laps3d_omp

        r = laps3d_omp.Run(n, CFG2)
        r.set_state(prim)
        if warmup:
            r.step(warmup)
        t0 = time.perf_counter()
        r.step(steps)
        el = time.perf_counter() - t0
        r.close()
        return (n**3 * steps / el, laps3d_omp.threads(),
                f"{warmup} warm-up + {steps} timed steps at {n}^3 (C++/OpenMP restatement, own radix-2 FFT, FP64)", "port")
    except (OSError, ValueError, subprocess.CalledProcessError):
        pass
    from oracle import laps3d

    o = laps3d.restart(n, CFG2, prim)
    for _ in range(warmup):
        o.vardt(); o.evolve(); o.time += o.dt; o.evolve_radius(o.time)
    t0 = time.perf_counter()
    for _ in range(steps):
        o.vardt(); o.evolve(); o.time += o.dt; o.evolve_radius(o.time)
    el = time.perf_counter() - t0
    return (n**3 * steps / el, laps3d._WORKERS,
            f"{warmup} warm-up + {steps} timed steps at {n}^3 (numpy + scipy.fft pocketfft)", "port")


def fp32_error(p, prim, steps, chunk=25):
    """Error of an FP32-transform run against the FP64 engine (which matches the oracle to
    1e-10) on the same workload: per-field relative L2, the invariants, the time and the shell
    spectra E_u(k), E_b(k) of every shell 1 <= k <= k_max / 2 (k_max = n/3, the 2/3 sphere).
    Both runs advance in chunks of `chunk` steps.  If the FP64 run collapses first - the CFL
    step below 1 % of its first value, or the dt floor - the statement is the last checkpoint
    before the collapse, and `collapse` records where it happened."""
    from laps_gb300 import ffi

    nshell = max(p.nx, p.ny, p.nz) // 3 + 1
    ctx = {}
    for name, mode in (("test", p.precision), ("fp64", ffi.PREC_FP64)):
        q = ffi.laps_params.from_buffer_copy(p)
        q.precision = mode
        r = ffi.Laps(q)
        r.upload_state(prim, primitive=True)
        r.set_time(0.0)
        ctx[name] = r

    def snapshot():
        out = {}
        for name, r in ctx.items():
            uu, _ = r.download_state()
            d = r.diagnostics()
            eu, eb = r.spectrum(nshell)
            t, dt = r.time()
            out[name] = (uu, np.array([d.e_kin, d.e_mag, d.h_cross, d.h_mag]), t, eu, eb, dt)
        return out

    done, dt0, good, collapse = 0, None, None, None
    while done < steps:
        k = min(chunk, steps - done)
        st = {name: r.step(k)[2] for name, r in ctx.items()}
        done += k
        t64, dt64 = ctx["fp64"].time()
        dt0 = dt0 or dt64
        if st["fp64"] != 0 or dt64 < 0.01 * dt0:
            collapse = {"step_checkpoint": done, "time": t64, "dt": dt64, "status": st["fp64"],
                        "note": "the FP64 run (the reference's algorithm) collapsed: CFL step below 1 % of its "
                                "first value or the dt floor; the statement is the last checkpoint before it"}
            break
        good = (done, snapshot())
    for r in ctx.values():
        r.close()
    if good is None:
        return {"steps": 0, "collapse": collapse}
    nsteps, snap = good
    a, b = snap["test"], snap["fp64"]
    rel = [float(np.linalg.norm(a[0][f] - b[0][f]) / max(np.linalg.norm(b[0][f]), 1e-300)) for f in range(8)]
    half = slice(1, (nshell - 1) // 2 + 1)
    out = {"steps": nsteps, "steps_requested": steps, "time": b[2], "field_rel_l2": rel, "max_field_rel_l2": max(rel),
           "invariants_rel": [float(v) for v in np.abs(a[1] - b[1]) / np.maximum(np.abs(b[1]), 1e-300)],
           "time_rel": abs(a[2] - b[2]) / b[2],
           "spectrum_shells": f"1..{half.stop - 1} (every shell up to k_max/2, k_max = n/3)"}
    for key, i in (("u", 3), ("b", 4)):
        ea, eb = a[i][half], b[i][half]
        relk = np.abs(ea - eb) / np.maximum(eb, 1e-300)
        out[f"spectrum_{key}_rel_by_shell"] = [float(f"{v:.3g}") for v in relk]
        out[f"spectrum_{key}_max_rel"] = float(relk.max())
        out[f"spectrum_{key}_max_abs_over_total"] = float(np.abs(ea - eb).max() / eb.sum())
    if collapse:
        out["collapse"] = collapse
    return out


def device_timed(p, prim, steps, warmup):
    """Steps of one context timed with CUDA events around every pass (state resident in HBM):
    (per-pass ms, total ms, status, info)."""
    from laps_gb300 import ffi

    g = ffi.Laps(p)
    g.upload_state(prim, primitive=True)
    g.set_time(0.0)
    g.step(warmup)
    info = g.info()
    pass_ms, total_ms, status = g.step_profiled(steps)
    g.close()
    return pass_ms, total_ms, status, info


def pinned_buffers(prim, local):
    """Page-locked host arrays (torch's pinned allocator) for the end-to-end leg, so the
    copies run at link speed; plain numpy arrays when torch cannot pin."""
    try:
        import torch

        torch.cuda.set_device(local)

        def pinned_array(shape):
            return torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()

        host_in = pinned_array(prim.shape)
        host_in[...] = prim
        return host_in, pinned_array((8,) + prim.shape[1:]), pinned_array((4,) + prim.shape[1:]), True
    except Exception:
        return (np.ascontiguousarray(prim), np.empty((8,) + prim.shape[1:]), np.empty((4,) + prim.shape[1:]), False)


def end_to_end(p, bufs, steps, npts, ws, sched=None):
    """The metric through the C-ABI with host buffers: upload of the primitive state from
    pinned host memory, `steps` laps_step(1) calls (each returns time, dt and status to the
    host), download of the final conserved state and primitives; host clock, max over ranks.
    One untimed pass of the same sequence warms the path first."""
    import ctypes

    from laps_gb300 import ffi

    lib = ffi.load()
    host_in, host_out, host_prim, pinned = bufs
    dptr = ctypes.POINTER(ctypes.c_double)
    ctx = ffi.Laps(p)
    if sched is not None:
        ctx.set_schedule(sched)
    ctx.upload_state(host_in, primitive=True)
    ctx.set_time(0.0)
    ctx.step(2)
    assert lib.laps_download_state(ctx.h, host_out.ctypes.data_as(dptr), host_prim.ctypes.data_as(dptr)) == 0
    barrier(ws)
    t0 = time.perf_counter()
    ctx.upload_state(host_in, primitive=True)
    ctx.set_time(0.0)
    t1 = time.perf_counter()
    for _ in range(steps):
        ctx.step(1)
    t2 = time.perf_counter()
    assert lib.laps_download_state(ctx.h, host_out.ctypes.data_as(dptr), host_prim.ctypes.data_as(dptr)) == 0
    t3 = time.perf_counter()
    ctx.close()
    e2e_s = barrier_max(t3 - t0, ws)
    return {"value": ws * npts * steps / e2e_s, "unit": "grid-point-steps/s",
            "h2d_bytes_per_step": host_in.nbytes / steps + 16,
            "d2h_bytes_per_step": (host_out.nbytes + host_prim.nbytes) / steps + 128,
            "pinned": pinned, "upload_s": t1 - t0, "steps_s": t2 - t1, "download_s": t3 - t2}


def roofline_of(pass_ms, steps, info, mode, n, workload):
    """Dominant pass of a mode: its algorithmic bytes (pass_bytes) over its average
    event-timed launch against the measured copy bandwidth, and the same figure for every
    pass; `traffic` is the ncu DRAM bytes of one launch of that pass (profiles/traffic.json,
    captured on a reduced grid and scaled by the planes processed), when present."""
    eS, eT = PRECISIONS[mode][2:4]
    pbf = pass_bytes_3di if WL["variant"] == 1 else pass_bytes
    pb = pbf(n, info.kx_keep, info.ky_keep, info.kz_keep, eS=eS, eT=eT) if not SHAPE else {k: 0 for k in PASS_NAMES[:5]}
    launches = steps * 3
    dom = max(range(5), key=lambda i: pass_ms[i])
    name = PASS_NAMES[dom]
    avg_ms = pass_ms[dom] / launches
    achieved = pb[name] / (avg_ms * 1e-3) / 1e9 if pb[name] else None
    peak, src = peaks()
    traffic = None
    tf = ROOT / "profiles" / "traffic.json"
    if tf.exists() and not SHAPE and n == WL["grid"]:
        try:
            traffic = json.loads(tf.read_text()).get(f"{workload}/{mode}", {}).get(name)
        except Exception:
            traffic = None
    roof = {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak if achieved else None, "peak_source": src, "traffic": traffic,
            "algorithmic_bytes_per_launch": pb[name]}
    per_pass = {PASS_NAMES[i]: {"gbs": pb[PASS_NAMES[i]] / (pass_ms[i] / launches * 1e-3) / 1e9,
                                "frac": pb[PASS_NAMES[i]] / (pass_ms[i] / launches * 1e-3) / 1e9 / peak}
                for i in range(5) if pb[PASS_NAMES[i]] and pass_ms[i] > 0}
    return roof, per_pass


# FP64 issue rate of this GPU's FP64 pipe: FMA/ADD instructions per second, measured with
# independent dependency chains on a GB300 (~1.6 per clock per SM at 2.07 GHz).  A flop rate
# counts an FMA as two.
FP64_INSTR_PER_S = 0.508e12


def fp64_roofline(pass_ms, steps, n, info):
    """The plain FP64 path against the FP64 pipe: the transform flops of pass C (24 real
    transforms of the x rows: 11 inverse, 13 forward, 2.5 n log2 n each, the benchFFT count)
    over its average launch, against 2 x the measured FP64 FMA issue rate."""
    c_ms = pass_ms[2] / (steps * 3)
    rows = n * n
    flops = 24 * rows * 2.5 * n * math.log2(n)
    achieved = flops / (c_ms * 1e-3) / 1e12
    peak = 2 * FP64_INSTR_PER_S / 1e12
    return {"bound": "fp64", "kernel": "C_x_flux", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak, "flops_per_launch": flops,
            "flop_count": "transforms only (2.5 n log2 n per real line); the flux physics adds more"}


def cufft_yardstick(n, pass_ms, steps, kind):
    """cuFFT (through torch.fft) on the same 256^3 fields: the transforms each pass does,
    unfused and unpruned, as batched R2C/C2R along x and C2C along y and z, in the pass's
    transform precision.  Outside the timed `value`; a yardstick for the hand-written
    passes, whose times include the physics, the RK update and the pruning."""
    import torch

    cdt = torch.complex64 if kind == "f32" else torch.complex128
    rdt = torch.float32 if kind == "f32" else torch.float64
    nh = n // 2 + 1
    dev = "cuda"
    # (pass, what cuFFT does): fields per launch of the compressible Hall + expanding-box stage
    jobs = {
        "A_inv_z": ("c2c_z", 10), "B_inv_y": ("c2c_y", 11), "C_x_flux": ("c2r_r2c_x", (11, 13)),
        "D_fwd_y": ("c2c_y", 13), "E_fwd_z_rk": ("c2c_z", 13),
    }
    out = {}
    spec = torch.randn((13, n, n, nh), dtype=cdt, device=dev)
    real = torch.randn((13, n, n, n), dtype=rdt, device=dev)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn, reps=5):
        fn()
        torch.cuda.synchronize()
        ev0.record()
        for _ in range(reps):
            fn()
        ev1.record()
        torch.cuda.synchronize()
        return ev0.elapsed_time(ev1) / reps

    for name, (op, nf) in jobs.items():
        if op == "c2c_z":
            ms = timed(lambda: torch.fft.ifft(spec[:nf], dim=1))
        elif op == "c2c_y":
            ms = timed(lambda: torch.fft.fft(spec[:nf], dim=2))
        else:
            ms = timed(lambda: torch.fft.irfft(spec[:nf[0]], n=n, dim=3)) + timed(lambda: torch.fft.rfft(real[:nf[1]], dim=3))
        ours = pass_ms[PASS_NAMES.index(name)] / (steps * 3)
        out[name] = {"cufft_ms": ms, "ours_ms": ours, "ours_over_cufft": ours / ms}
    del spec, real
    torch.cuda.empty_cache()
    tot_c = sum(v["cufft_ms"] for v in out.values())
    tot_o = sum(v["ours_ms"] for v in out.values())
    return {"library": f"cuFFT via torch.fft (torch {torch.__version__})", "precision": kind, "per_stage": out,
            "stage_cufft_ms": tot_c, "stage_ours_ms": tot_o, "ours_over_cufft": tot_o / tot_c,
            "note": "cuFFT: transforms only, all modes; ours: the fused passes with physics, RK update and dealias "
                    "pruning"}


def bf16_peak():
    try:
        d = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
        return float(d["bf16_tflops"]), "measured"
    except Exception:
        return 1900.0, "fallback"


def closure_conv_bench(n=128, reps=20):
    """The closure net's tensor-core convolutions on the coarse grid (n^3, periodic): one
    32 -> 32 channel 3x3x3 layer forward with GELU, its input-gradient and its weight-gradient
    kernels, timed with CUDA events on the stream they run on; TFLOP/s = 2 x voxels x 27 x 32 x
    32 per kernel over its average time, against the dense BF16 peak."""
    import torch

    from laps_gb300 import closure

    dev = "cuda"
    g = torch.Generator(device=dev).manual_seed(4)
    x = torch.randn((n, n, n + 2, 32), device=dev, generator=g).to(torch.bfloat16)
    dz = torch.randn((n, n, n + 2, 32), device=dev, generator=g).to(torch.bfloat16)
    w = torch.randn((32, 32, 3, 3, 3), device=dev, generator=g) * 0.05
    b = torch.zeros(32, device=dev)
    pk, pkf = closure.pack(w, 32, 32), closure.pack(w, 32, 32, flip=True)
    y = torch.empty_like(x)
    zp = torch.empty_like(x)
    runs = {
        "forward_gelu": lambda: closure.conv3(x, pk, 32, bias=b, act=1, zpre=zp, out=y),
        "input_gradient": lambda: closure.conv3(dz, pkf, 32, act=2, gate=zp, out=y),
        "weight_gradient": lambda: closure.wgrad(x, dz, 32, 32),
    }
    flops = 2.0 * n**3 * 27 * 32 * 32
    peak, src = bf16_peak()
    out = {"grid": f"{n}^3", "channels": "32 -> 32", "flops_per_kernel": flops, "peak_tflops": peak,
           "peak_source": src}
    s = torch.cuda.current_stream()
    for name, fn in runs.items():
        for _ in range(3):
            fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for _ in range(reps):
            fn()
        e1.record(s)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        tf = flops / (ms * 1e-3) / 1e12
        out[name] = {"ms": ms, "tflops": tf, "frac": tf / peak}
    out["status"] = closure.status()
    # algorithmic bytes of the forward layer: input read once, output and pre-activation written
    fwd_bytes = 3 * n * n * (n + 2) * 32 * 2
    out["forward_gelu"]["hbm_gbs"] = fwd_bytes / (out["forward_gelu"]["ms"] * 1e-3) / 1e9
    return out


def measure_mode(mode, p0, prim, args, npts, bufs, ws, local, with_clocks=False):
    """One arithmetic mode on the workload: device-timed steps (CUDA events around every pass,
    state resident in HBM), the graph path, the end-to-end leg, and the roofline figures."""
    from laps_gb300 import ffi

    from laps_gb300 import autotune

    q = ffi.laps_params.from_buffer_copy(p0)
    q.precision = PRECISIONS[mode][0]
    g = ffi.Laps(q)
    g.upload_state(prim, primitive=True)
    g.set_time(0.0)
    g.step(max(args.warmup, 3))
    tuned = None
    if not args.no_tune:  # the execution schedule (outside the timed region; cached on disk)
        tuned = autotune.tune(g, steps=2)
        g.upload_state(prim, primitive=True)  # the timed steps start from the same state
        g.set_time(0.0)
        g.step(max(args.warmup, 3))
    info = g.info()
    barrier(ws)
    clk = Clocks(local) if with_clocks else None
    if clk:
        clk.__enter__()
    pass_ms, total_ms, status = g.step_profiled(args.steps)
    if clk:
        clk.__exit__()
    barrier(ws)
    tmax = barrier_max(total_ms, ws)
    t0 = time.perf_counter()
    g.step(args.steps)  # the graph path (what laps_step replays), same state continuing
    graph_ms = (time.perf_counter() - t0) * 1e3 / args.steps
    g.close()
    n = N_GRID
    roof, per_pass = roofline_of(pass_ms, args.steps, info, mode, n, args.workload)
    res = {"value": ws * npts * args.steps / (tmax * 1e-3), "ms_per_step": tmax / args.steps, "status": status,
           "dtype": PRECISIONS[mode][1], "graph_ms_per_step": graph_ms,
           "pass_ms_per_step": {PASS_NAMES[i]: pass_ms[i] / args.steps for i in range(6)},
           "roofline": roof, "passes_hbm": per_pass,
           "e2e": end_to_end(q, bufs, args.steps, npts, ws, None if args.no_tune else tuned["bits"]),
           "_info": info, "_pass_ms": pass_ms}
    if tuned is not None:
        res["schedule"] = {"bits": tuned["bits"], "from_cache": tuned["from_cache"],
                           "candidates_ms_per_step": {str(b): round(t, 4) for b, t in tuned["times_ms"].items()}}
    if clk:
        res["clocks"] = clk.summary()
    if mode == "fp64" and not SHAPE and WL["variant"] == 0:
        res["fp64_roofline"] = fp64_roofline(pass_ms, args.steps, n, info)
    return res


def run_ensemble(args):
    """The batched 2-D ensemble: 64 independent 2-D compressible Hall-MHD runs with uneven
    grids (128^2 .. 1024^2) and per-member eta, nu, d_i and field angle (seed 3), advanced by
    one graph per step.  value = sum of member grid points x steps / wall time of K steps
    (host clock around laps_batch_step, whose only host work is K graph launches and one
    wait); e2e adds the uploads of every member's primitive state and the downloads."""
    from laps_gb300 import ffi
    from laps_gb300.ic import ensemble_2d, member_ic

    ms = ensemble_2d(nmembers=args.members, seed=3)
    prec = PRECISIONS[args.precision][0]
    plist = [ffi.params(precision=prec, **m["kw"]) for m in ms]
    prims = [member_ic(m) for m in ms]
    npts = sum(m["n"] ** 2 for m in ms)
    b = ffi.Batch(plist)
    for i, prim in enumerate(prims):
        b.members[i].upload_state(prim, primitive=True)
        b.members[i].set_time(0.0)
    schedules = {}
    if not args.no_tune:  # one tuning per member kind (grid, precision, ...), then the cache
        from laps_gb300 import autotune

        cache = autotune.load_cache()
        for i, prim in enumerate(prims):
            m = b.members[i]
            r = autotune.tune(m, steps=2, cache=cache)
            schedules[r["key"]] = r["bits"]
            if not r["from_cache"]:
                m.upload_state(prim, primitive=True)
                m.set_time(0.0)
        autotune.save_cache(cache)
    b.step(max(args.warmup, 3))
    with Clocks(0) as clk:
        t0 = time.perf_counter()
        _, _, st = b.step(args.steps)
        el = time.perf_counter() - t0
    value = npts * args.steps / el
    # e2e: uploads, K steps, downloads
    t0 = time.perf_counter()
    for i, prim in enumerate(prims):
        b.members[i].upload_state(prim, primitive=True)
        b.members[i].set_time(0.0)
    b.step(args.steps)
    out = [b.members[i].download_state() for i in range(len(ms))]
    e2e_s = time.perf_counter() - t0
    h2d = sum(p.nbytes for p in prims) / args.steps
    d2h = sum(u.nbytes + q.nbytes for u, q in out) / args.steps
    sizes = {}
    for m in ms:
        sizes[m["n"]] = sizes.get(m["n"], 0) + 1
    # CPU baseline: the 2-D numpy restatement on one member of each grid size, 1 warm-up + 2
    # timed steps each (a bounded sample; the same metric over the sampled members)
    cpu = None
    if not args.no_cpu:
        from oracle import laps3d

        pts, cpu_s, seen = 0, 0.0, set()
        for m, prim in zip(ms, prims):
            if m["n"] in seen:
                continue
            seen.add(m["n"])
            kw = {k: v for k, v in m["kw"].items() if k not in ("variant", "nx", "ny", "nz")}
            o = laps3d.restart2d(m["n"], kw, prim)
            o.dt = 0.0
            o.step()
            t0 = time.perf_counter()
            for _ in range(2):
                o.step()
            cpu_s += time.perf_counter() - t0
            pts += 2 * m["n"] ** 2
        cpu = {"value": pts / cpu_s, "unit": "grid-point-steps/s", "cores": laps3d._WORKERS, "kind": "port",
               "sample": f"one member of each grid size {sorted(seen)}, 1 warm-up + 2 timed steps each "
                         f"(numpy + scipy.fft 2-D restatement)"}
    # whole-step roofline: the algorithmic bytes of every member's three stages (pass_bytes_2d)
    # over the timed step, against the measured copy bandwidth; kernel launches from each
    # member's own count per step
    eS, eT = PRECISIONS[args.precision][2:4]
    step_bytes, launches = 0, 0
    for m in b.members:
        inf = m.info()
        step_bytes += 3 * sum(pass_bytes_2d(m.p.nx, inf.kx_keep, inf.ky_keep, eS=eS, eT=eT).values())
        launches += inf.kernels_per_step
    peak, src = peaks()
    achieved = step_bytes / (el / args.steps) / 1e9
    line = {
        "metric": "grid-point-steps/s of a 64-member 2-D Hall-MHD ensemble", "value": value, "unit": "grid-point-steps/s",
        "n_gpus": 1, "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": el / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": PRECISIONS[args.precision][1],
        "data": "synthetic (seeded random-phase spectra 1<=|k|<=8, rms 0.3, per-member seeds)",
        "config": {"workload": f"{len(ms)} independent 2-D compressible Hall-MHD runs, grids {sorted(sizes.items())}",
                   "grid_points_per_step": npts, "dealias": "2/3 circle", "cfl": 0.4, "vardt": "every 20 steps",
                   "timing": "host clock around laps_batch_step (one graph launch per step)",
                   "l2": "inputs larger than L2"},
        "status_nonzero_members": int((st != 0).sum()),
        "schedules": schedules,
        "cpu_baseline": cpu,
        "gpu_launches": launches * args.steps,
        "roofline": {"bound": "hbm", "kernel": "whole step (every pass of every member)", "achieved": achieved,
                     "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_source": src, "traffic": None,
                     "algorithmic_bytes_per_step": step_bytes},
        "e2e": {"value": npts * args.steps / e2e_s, "unit": "grid-point-steps/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)
    b.close()
    return 0


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    k = max(1, args.steps if args.ref_steps <= 0 else min(args.steps, args.ref_steps))
    w = args.warmup
    v, cores, sample, kind = cpu_sample(k, w)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "grid-point-steps/s", "n_gpus": args.gpus,
        "steps": k, "warmup": w, "ms_per_step": N_GRID**3 / v * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded random-phase spectrum)",
        "config": {"workload": WORKLOAD, "grid": N_GRID, "variant": "3DC", "hall": 0.05, "expanding_box": "Ur0/R0=0.01",
                   "dealias": "2/3 sphere", "l2": "inputs larger than L2"},
        "cpu_baseline": {"value": v, "unit": "grid-point-steps/s", "cores": cores, "kind": kind, "sample": sample},
        "e2e": {"value": v, "unit": "grid-point-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
    from laps_gb300 import ffi

    n = N_GRID
    prim = initial_state()
    nx, ny, nz = SHAPE if SHAPE else (n, n, n)
    npts = nx * ny * nz
    p = ffi.params(nx=nx, ny=ny, nz=nz, precision=PRECISIONS[args.precision][0], device=local,
                   variant=WL["variant"], **WL["kw"])
    bufs = pinned_buffers(prim, local)
    head = measure_mode(args.precision, p, prim, args, npts, bufs, ws, local, with_clocks=True)
    info = head.pop("_info")
    pass_ms = head.pop("_pass_ms")
    # ---- the other arithmetic modes on the same workload (rank 0 of a single run)
    plain = {}
    if not args.no_plain and rank == 0 and ws == 1:
        for mode in ("fp32", "dd", "fp64"):
            if mode == args.precision:
                continue
            r = measure_mode(mode, p, prim, args, npts, bufs, ws, local)
            r.pop("_info"), r.pop("_pass_ms")
            plain[mode] = r
    line = {
        "metric": METRIC, "value": head["value"], "unit": "grid-point-steps/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": PRECISIONS[args.precision][1],
        "data": WL["data"],
        "config": dict({"workload": WORKLOAD, "grid": n, "precision": args.precision}, **WL["desc"],
                       parallelism=f"replicas x{ws}", l2=f"inputs larger than L2 ({info.device_bytes / 1e9:.0f} GB working set)"),
        "gpu_launches": args.steps * info.kernels_per_step,
        "status": head["status"],
        "graph_ms_per_step": head["graph_ms_per_step"],
        "pass_ms_per_step": head["pass_ms_per_step"],
        "roofline": head["roofline"],
        "passes_hbm": head["passes_hbm"],
        "e2e": head["e2e"],
        "clocks": head["clocks"],
    }
    if "schedule" in head:
        line["config"]["schedule"] = head["schedule"]
    if plain:
        line["plain"] = plain
        line["vs_plain"] = {k: head["value"] / v["value"] for k, v in plain.items()}
    if rank == 0 and ws == 1 and not SHAPE and not args.no_cufft and WL["variant"] == 0:
        try:
            line["cufft_yardstick"] = cufft_yardstick(n, pass_ms, args.steps,
                                                      "f32" if args.precision.startswith("fp32") else "f64")
        except Exception as e:  # torch without CUDA, or out of memory: say so
            line["cufft_yardstick"] = {"unavailable": f"{type(e).__name__}: {e}"[:200]}
    if rank == 0 and ws == 1 and not SHAPE and not args.no_closure:
        try:
            line["closure_conv"] = closure_conv_bench()
        except Exception as e:
            line["closure_conv"] = {"unavailable": f"{type(e).__name__}: {e}"[:200]}
    if args.precision.startswith("fp32") and not SHAPE and not args.no_err and rank == 0:
        line["error_vs_fp64"] = fp32_error(p, prim, args.err_steps)
        if WL["variant"] == 0:
            # The workload's recipe (rms 0.5 on a beta 0.2 background) is far from pressure
            # balance: its magnetic-pressure fluctuations drive the pressure negative and the
            # FP64 run collapses to the dt floor near t = 0.28 (step ~250 at 256^3) under the
            # reference's own algorithm.  The full step count is stated on the same recipe at
            # rms 0.1, which stays pressure-positive.
            from laps_gb300.ic import turbulence_ic

            low = turbulence_ic(N_GRID, kmin=1, kmax=8, alpha=-1.0, rms_u=0.1, rms_b=0.1, seed=1)
            e = fp32_error(p, low, args.err_steps)
            e["workload"] = "the same recipe at rms 0.1 (pressure stays positive for the whole run)"
            line["error_vs_fp64_rms01"] = e
    if rank == 0 and ws == 1 and not args.no_cpu and WL["variant"] == 0:
        v, cores, sample, kind = cpu_sample(args.cpu_steps, 1)
        line["cpu_baseline"] = {"value": v, "unit": "grid-point-steps/s", "cores": cores, "kind": kind, "sample": sample}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    return 0


def main():
    global N_GRID, WORKLOAD, WL
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp32_f64", choices=list(PRECISIONS),
                    help="headline mode: fp32_f64 (FP32 transforms and products, FP64 state / RK / CFL / "
                         "diagnostics: the FP32-FFT option), fp32 (the same with a float-float state), dd, fp64")
    ap.add_argument("--workload", default="c3d256", choices=["c3d256", "c3di512", "ens2d"],
                    help="c3d256: the 3-D Hall + expanding-box case (headline); c3di512: the 3-D incompressible "
                         "FP32-vs-FP64 study at 512^3; ens2d: the 2-D ensemble")
    ap.add_argument("--members", type=int, default=64, help="ensemble members (--workload ens2d)")
    ap.add_argument("--no-plain", action="store_true", dest="no_plain",
                    help="skip timing the plain float-float and FP64 paths beside the headline mode")
    ap.add_argument("--err-steps", type=int, default=500, dest="err_steps",
                    help="steps of the FP32-vs-FP64 error check of the fp32 modes (the workload's step count)")
    ap.add_argument("--no-cufft", action="store_true", dest="no_cufft", help="skip the cuFFT yardstick")
    ap.add_argument("--no-tune", action="store_true", dest="no_tune",
                    help="skip the schedule autotuner (laps_gb300/autotune.py) and run the default schedule")
    ap.add_argument("--no-closure", action="store_true", dest="no_closure",
                    help="skip the closure convolutions' tensor-core measurement")
    ap.add_argument("--cpu-steps", type=int, default=5, dest="cpu_steps",
                    help="timed steps of the CPU baseline (after one warm-up step)")
    ap.add_argument("--no-err", action="store_true", dest="no_err")
    ap.add_argument("--ref-steps", type=int, default=0, dest="ref_steps",
                    help="cap on the timed steps of --impl reference (0: the same --steps as our arm)")
    ap.add_argument("--no-cpu", action="store_true", dest="no_cpu")
    ap.add_argument("--grid", type=int, default=256, help="grid size n (n^3); the headline workload is 256")
    ap.add_argument("--shape", default=None, help="nx,ny,nz of a reduced profiling case (overrides --grid)")
    args = ap.parse_args()
    global SHAPE
    if args.workload in WORKLOADS:
        WL = WORKLOADS[args.workload]
        if args.grid == 256 and WL["grid"] != 256:
            args.grid = WL["grid"]
        N_GRID = WL["grid"]
        WORKLOAD = f"{WL['label']}, {N_GRID}^3"
    if args.shape:
        SHAPE = tuple(int(v) for v in args.shape.split(","))
        WORKLOAD = f"{WL['label']}, {args.shape} (reduced case)"
    if args.grid != N_GRID:
        N_GRID = args.grid
        WORKLOAD = f"{WL['label']}, {N_GRID}^3 (reduced case)"
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "ens2d":
        return run_ensemble(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
