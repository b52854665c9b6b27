"""GPU parity of the 3-D incompressible and 2-D compressible variants against the oracle,
through the C-ABI (FP64 and float-float)."""
import math

import numpy as np
import pytest

from laps_gb300 import ffi
from laps_gb300.ic import alfven_wave_ic, turbulence_ic
from oracle import laps3d

from pairs import rel_l2, state_floor

pytestmark = pytest.mark.gpu
PRECS = [ffi.PREC_FP64, ffi.PREC_DD]
PREC_ID = ["fp64", "dd"]

I_CASES = {
    "plain": dict(if_resis=1, resistivity=2e-4, if_visc=1, viscosity=2e-4, dealias_option=1, cfl=0.4),
    "hall_ebm": dict(if_resis=1, resistivity=5e-4, if_visc=1, viscosity=5e-4, dealias_option=1, cfl=0.4, if_Hall=1,
                     ion_inertial_length=0.05, if_AEB=1, radius0=30.0, Ur0=0.3),
    "explicit_filter": dict(if_resis=1, resistivity=1e-3, if_resis_exp=1, if_visc=1, viscosity=1e-3, if_visc_exp=1,
                            dealias_option=2, cfl=0.3),
    "corot": dict(dealias_option=1, cfl=0.4, if_AEB=1, radius0=30.0, Ur0=0.3, if_corotating=1, corotating_angle=0.4,
                  if_resis=1, resistivity=5e-4, if_visc=1, viscosity=5e-4),
}
D_CASES = {
    "hall": dict(dealias_option=1, cfl=0.4, if_Hall=1, ion_inertial_length=0.05, if_resis=1, resistivity=1e-3,
                 if_visc=1, viscosity=1e-3),
    "zradial_square": dict(dealias_option=3, cfl=0.4, if_AEB=1, radius0=30.0, Ur0=0.3, if_z_radial=1),
    "ebm_plain": dict(dealias_option=1, cfl=0.4, if_AEB=1, radius0=30.0, Ur0=0.3, if_Hall=1, ion_inertial_length=0.03),
    "filter_explicit_limit": dict(dealias_option=2, cfl=0.4, if_resis=1, resistivity=1e-3, if_resis_exp=1,
                                  if_limit_dt_increase=1, if_conserve_background=1),
    "corot": dict(dealias_option=1, cfl=0.4, if_AEB=1, radius0=30.0, Ur0=0.3, if_corotating=1, corotating_angle=0.3),
}


def start_i(n, kw, prim, prec, t0=0.0):
    o = laps3d.restart3di(n, kw, prim, t0)
    g = ffi.Laps(ffi.params(nx=n, ny=n, nz=n, variant=ffi.VARIANT_3DI, precision=prec, **kw))
    g.upload_state(prim, primitive=True)
    g.set_time(t0)
    return o, g


def start_2d(shape, kw, prim, prec, t0=0.0):
    o = laps3d.restart2d(shape, kw, prim, t0)
    g = ffi.Laps(ffi.params(nx=shape[0], ny=shape[1], nz=1, variant=ffi.VARIANT_2DC, precision=prec, **kw))
    g.upload_state(prim, primitive=True)
    g.set_time(t0)
    return o, g


@pytest.mark.parametrize("prec", PRECS, ids=PREC_ID)
@pytest.mark.parametrize("case", list(I_CASES))
def test_incompressible_stage(prec, case):
    kw = I_CASES[case]
    prim = turbulence_ic(32, seed=12, kmax=5, rms_u=0.4, rms_b=0.4, p0=1.0)
    o, g = start_i(32, kw, prim, prec, t0=1.0 if kw.get("if_AEB") else 0.0)
    o.dt = 0.0
    assert abs(g.vardt() - o.vardt()) <= 1e-13 * o.dt
    o.stage(1)
    g.rk_stage(1)
    uu, _ = g.download_state()
    assert rel_l2(uu, o.uu, state_floor(o.uu)).max() < 1e-12
    uf = g.download_spectral()
    assert np.abs(uf - o.uf).max() <= 1e-12 * np.abs(o.uf).max()


@pytest.mark.parametrize("prec", PRECS, ids=PREC_ID)
@pytest.mark.parametrize("case", list(I_CASES))
def test_incompressible_steps(prec, case):
    kw = I_CASES[case]
    prim = turbulence_ic(32, seed=13, kmax=5, rms_u=0.4, rms_b=0.4, p0=1.0)
    o, g = start_i(32, kw, prim, prec)
    o.dt = 0.0
    for _ in range(8):
        o.step()
    t, dt, st = g.step(8)
    assert st == 0 and abs(t - o.time) <= 1e-12 * o.time
    uu, pr = g.download_state()
    assert rel_l2(uu, o.uu, state_floor(o.uu)).max() < 1e-11
    d = g.diagnostics()
    db, dv = o.div_maxima()
    # div B is zero up to round-off here (both sides ~1e-14); div V is not (expanding box)
    assert abs(d.max_divB_real - db) <= 1e-9 * db + 1e-12
    assert abs(d.max_divV_real - dv) <= 1e-9 * dv + 1e-12
    assert np.allclose([d.e_kin, d.e_mag, d.h_cross, d.h_mag], o.invariants(), rtol=1e-10, atol=1e-14)


@pytest.mark.parametrize("prec", PRECS, ids=PREC_ID)
def test_incompressible_alfven_wave(prec):
    n, eta = 16, 1e-2
    kw = dict(if_resis=1, resistivity=eta, if_visc=1, viscosity=eta, dealias_option=1, cfl=0.05)
    o, g = start_i(n, kw, alfven_wave_ic(n, db0=0.1), prec)
    t, dt, st = g.step(40)
    uu, _ = g.download_state()
    x = np.arange(n) * (2 * math.pi / n)
    dec = math.exp(-eta * t)
    assert np.abs(uu[6] + 0.1 * np.sin(x - t) * dec).max() < 1e-5
    assert np.abs(uu[5] + 0.1 * np.cos(x - t) * dec).max() < 1e-5


@pytest.mark.parametrize("prec", PRECS, ids=PREC_ID)
@pytest.mark.parametrize("case", list(D_CASES))
def test_2d_steps(prec, case):
    kw = D_CASES[case]
    shape = (64, 32)
    prim = turbulence_ic((64, 32, 1), seed=14, kmax=6, rms_u=0.3, rms_b=0.3)
    o, g = start_2d(shape, kw, prim, prec)
    o.dt = 0.0
    for _ in range(45):  # crosses two vardt cadence points (every 20 steps)
        o.step()
    t, dt, st = g.step(45)
    assert st == 0
    assert abs(t - o.time) <= 1e-12 * o.time and abs(dt - o.dt) <= 1e-12 * o.dt
    uu, _ = g.download_state()
    assert rel_l2(uu, o.uu, state_floor(o.uu)).max() < 1e-11
    d = g.diagnostics()
    assert np.allclose([d.e_kin, d.e_mag, d.h_cross, d.h_mag], o.invariants(), rtol=1e-10, atol=1e-14)
    assert abs(d.max_divB - o.calc_max_divB()) <= 1e-9 * o.calc_max_divB() + 1e-12  # both round-off here


@pytest.mark.parametrize("prec", PRECS, ids=PREC_ID)
def test_2d_alfven_wave(prec):
    n, eta = 32, 1e-2
    kw = dict(if_resis=1, resistivity=eta, if_visc=1, viscosity=eta, dealias_option=1, cfl=0.05, dstep_calcdt=1)
    o, g = start_2d((n, n), kw, alfven_wave_ic((n, n, 1), db0=0.1), prec)
    t, dt, st = g.step(40)
    uu, _ = g.download_state()
    x = np.arange(n) * (2 * math.pi / n)
    dec = math.exp(-eta * t)
    assert np.abs(uu[6] + 0.1 * np.sin(x - t) * dec).max() < 1e-5


@pytest.mark.parametrize("prec", PRECS + [ffi.PREC_FP32], ids=PREC_ID + ["fp32"])
@pytest.mark.parametrize("shape", [(32, 1024), (1024, 16)], ids=["ny1024", "nx1024"])
def test_2d_long_lines(prec, shape):
    """1024-point lines: 2-D y columns of 16-byte elements keep one tile in shared memory (the
    second in registers), 1024-point x rows run one row per block."""
    kw = D_CASES["hall"]
    prim = turbulence_ic((shape[0], shape[1], 1), seed=15, kmax=6, rms_u=0.3, rms_b=0.3)
    o, g = start_2d(shape, kw, prim, prec)
    o.dt = 0.0
    for _ in range(3):
        o.step()
    t, dt, st = g.step(3)
    assert st == 0
    tol = 1e-5 if prec == ffi.PREC_FP32 else 1e-11
    assert abs(dt - o.dt) <= tol * o.dt
    uu, _ = g.download_state()
    assert rel_l2(uu, o.uu, state_floor(o.uu)).max() < tol
