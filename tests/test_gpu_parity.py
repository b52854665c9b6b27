"""GPU parity against the oracle (CPU restatement of the reference), through the C-ABI.

Tolerances: FP64 and float-float runs must match the oracle's FP64 run to <= 1e-10
relative L2 in every field (the bar for 100 steps); shorter runs use tighter bounds stated
per test.  Transforms alone must agree to round-off (<= 1e-13 relative).
"""
import math

import numpy as np
import pytest

from laps_gb300 import ffi
from oracle.laps3d import forward_3d

from pairs import CONFIG1, CONFIG2, alfven, rel_l2, start_pair, state_floor, turb

pytestmark = pytest.mark.gpu

PRECS = [ffi.PREC_FP64, ffi.PREC_DD]
PREC_ID = ["fp64", "dd"]


@pytest.mark.parametrize("prec", PRECS, ids=PREC_ID)
@pytest.mark.parametrize("n", [16, (32, 16, 8), (16, 32, 64)])
def test_upload_download_roundtrip(prec, n):
    prim = turb(n, seed=3)
    o, g = start_pair(n, CONFIG1, prim, prec)
    uu, pr = g.download_state()
    assert rel_l2(uu, o.uu, state_floor(o.uu)).max() < 1e-13
    assert rel_l2(pr, o.uu_prim, state_floor(o.uu_prim)).max() < 1e-12


@pytest.mark.parametrize("prec", PRECS, ids=PREC_ID)
@pytest.mark.parametrize("n", [16, (32, 16, 8), (64, 32, 16)])
def test_forward_transform_matches_oracle(prec, n):
    prim = turb(n, seed=4)
    o, g = start_pair(n, CONFIG1, prim, prec)
    uf = g.download_spectral()
    ref = forward_3d(o.uu)
    err = np.abs(uf - ref).max() / np.abs(ref).max()
    assert err < 1e-14


@pytest.mark.parametrize("prec", PRECS, ids=PREC_ID)
@pytest.mark.parametrize("case", ["config1", "config2", "filter", "explicit", "corot"])
def test_one_stage(prec, case):
    n = 32
    kw = {
        "config1": CONFIG1,
        "config2": CONFIG2,
        "filter": dict(CONFIG1, dealias_option=2),
        "explicit": dict(CONFIG2, if_resis_exp=1, if_visc_exp=1, if_conserve_background=1),
        "corot": dict(CONFIG2, if_corotating=1, corotating_angle=0.3),
    }[case]
    prim = turb(n, seed=5, kmax=6, rms_u=0.4, rms_b=0.4)
    o, g = start_pair(n, kw, prim, prec, t0=1.5 if kw.get("if_AEB") else 0.0)
    o.dt = 0.0
    dto = o.vardt()
    dtg = g.vardt()
    assert abs(dtg - dto) <= 1e-13 * dto
    o.stage(1)
    g.rk_stage(1)
    uu, pr = g.download_state()
    err = rel_l2(uu, o.uu, state_floor(o.uu))
    assert err.max() < 1e-12, err
    uf = g.download_spectral()
    assert np.abs(uf - o.uf).max() <= 1e-12 * np.abs(o.uf).max()


@pytest.mark.parametrize("prec", PRECS, ids=PREC_ID)
@pytest.mark.parametrize("case", ["config1", "config2", "filter", "corot"])
def test_steps(prec, case):
    n = 32
    kw = {
        "config1": CONFIG1,
        "config2": CONFIG2,
        "filter": dict(CONFIG1, dealias_option=2),
        "corot": dict(CONFIG2, if_corotating=1, corotating_angle=0.3),
    }[case]
    prim = turb(n, seed=6, kmax=6, rms_u=0.4, rms_b=0.4)
    o, g = start_pair(n, kw, prim, prec)
    o.dt = 0.0
    nsteps = 10
    times = []
    for _ in range(nsteps):
        o.vardt()
        o.evolve()
        o.time += o.dt
        o.evolve_radius(o.time)
        times.append(o.time)
    t, dt, status = g.step(nsteps)
    assert status == 0
    assert abs(t - times[-1]) <= 1e-12 * times[-1]
    uu, pr = g.download_state()
    err = rel_l2(uu, o.uu, state_floor(o.uu))
    assert err.max() < 1e-11, err


@pytest.mark.parametrize("prec", PRECS, ids=PREC_ID)
def test_config1_100_steps(prec):
    """The 64^3 plain case for 100 steps: every field within 1e-10 relative L2, and the
    energy / cross-helicity / magnetic-helicity histories within 1e-9."""
    n = 64
    prim = turb(n, seed=0, kmin=1, kmax=4, alpha=-1.0, rms_u=0.3, rms_b=0.3)
    o, g = start_pair(n, CONFIG1, prim, prec)
    o.dt = 0.0
    hist_o, hist_g = [], []
    for k in range(100):
        o.vardt()
        o.evolve()
        o.time += o.dt
        o.evolve_radius(o.time)
        if k % 25 == 24:
            hist_o.append(o.invariants())
    for k in range(4):
        g.step(25)
        d = g.diagnostics()
        hist_g.append(np.array([d.e_kin, d.e_mag, d.h_cross, d.h_mag]))
    uu, pr = g.download_state()
    err = rel_l2(uu, o.uu, state_floor(o.uu))
    assert err.max() < 1e-10, err
    ho, hg = np.array(hist_o), np.array(hist_g)
    herr = np.abs(hg - ho) / np.maximum(np.abs(ho), 1e-12)
    assert herr.max() < 1e-9, herr


@pytest.mark.parametrize("prec", PRECS, ids=PREC_ID)
def test_diagnostics_match_oracle(prec):
    n = 32
    prim = turb(n, seed=7)
    o, g = start_pair(n, CONFIG2, prim, prec, t0=2.0)
    o.dt = 0.0
    o.vardt()
    o.evolve()
    g.vardt()
    for irk in (1, 2, 3):
        g.rk_stage(irk)
    d = g.diagnostics()
    ave, rms, ru2 = o.calc_rms()
    assert np.allclose(np.array(d.uu_ave[:]), ave, rtol=1e-12, atol=1e-14)
    assert np.allclose(np.array(d.uu_rms[:]), rms, rtol=1e-9, atol=1e-14)
    assert np.allclose(np.array(d.rho_u2[:]), ru2, rtol=1e-10, atol=1e-14)
    assert abs(d.max_divB - o.calc_max_divB()) <= 1e-10 * max(o.calc_max_divB(), 1e-12) + 1e-15
    inv = o.invariants()
    assert np.allclose([d.e_kin, d.e_mag, d.h_cross, d.h_mag], inv, rtol=1e-11, atol=1e-14)


@pytest.mark.parametrize("prec", PRECS, ids=PREC_ID)
def test_alfven_wave_known_answer(prec):
    """ipert=1: the circularly polarised Alfven wave travels at v_A = 1 and decays as
    exp(-eta k^2 t) with eta = nu (mhdinit.f90:328-342).  The GPU run matches the oracle to
    round-off, and both match the exact solution within RK3's truncation error (the
    measured error at this dt is 2.2e-6 of an amplitude 0.1)."""
    n, eta = 16, 1e-2
    kw = dict(if_resis=1, resistivity=eta, if_visc=1, viscosity=eta, dealias_option=1, cfl=0.05)
    prim = alfven(n, db0=0.1)
    o, g = start_pair(n, kw, prim, prec)
    t, dt, st = g.step(40)
    o.dt = 0.0
    for _ in range(40):
        o.vardt(); o.evolve(); o.time += o.dt; o.evolve_radius(o.time)
    assert abs(t - o.time) <= 1e-13 * t
    uu, _ = g.download_state()
    assert rel_l2(uu, o.uu, state_floor(o.uu)).max() < 1e-12
    x = np.arange(n) * (2 * math.pi / n)
    dec = math.exp(-eta * t)
    bz = -0.1 * np.sin(x - t) * dec
    by = -0.1 * np.cos(x - t) * dec
    assert np.abs(uu[6] - bz[None, None, :]).max() < 1e-5
    assert np.abs(uu[5] - by[None, None, :]).max() < 1e-5
    assert np.abs(uu[4] - 1.0).max() < 1e-12


@pytest.mark.parametrize("prec", PRECS, ids=PREC_ID)
def test_nan_is_reported(prec):
    n = 16
    prim = turb(n, seed=8)
    prim[0, 3, 4, 5] = np.nan  # injected on the host before upload
    _, g = start_pair(n, CONFIG1, prim, prec)
    t, dt, status = g.step(1)
    assert status & ffi.LAPS_STATUS_NAN


@pytest.mark.parametrize("prec", PRECS, ids=PREC_ID)
def test_dt_floor_stops_without_stepping(prec):
    n = 16
    prim = turb(n, seed=9)
    kw = dict(CONFIG1, cfl=1e-9)
    o, g = start_pair(n, kw, prim, prec)
    before = g.download_spectral()
    t, dt, status = g.step(3)
    assert status & ffi.LAPS_STATUS_DT_FLOOR
    assert t == 0.0 and dt < 1e-8
    after = g.download_spectral()
    assert np.array_equal(before, after)


@pytest.mark.parametrize("prec", [ffi.PREC_DD, ffi.PREC_FP64], ids=["dd", "fp64"])
@pytest.mark.parametrize("shape", [(512, 16, 8), (16, 512, 8), (16, 8, 512)], ids=["x512", "y512", "z512"])
def test_long_lines_one_step(prec, shape):
    """512-point lines along each axis (the 512^3 workloads' transform sizes): one step of the
    Hall + expanding-box case within 1e-12."""
    prim = turb(shape, seed=31, kmax=4, rms_u=0.3, rms_b=0.3)
    o, g = start_pair(shape, CONFIG2, prim, prec)
    o.dt = 0.0
    o.vardt(); o.evolve(); o.time += o.dt; o.evolve_radius(o.time)
    t, dt, status = g.step(1)
    assert status == 0 and abs(dt - o.dt) <= 1e-13 * o.dt
    uu, _ = g.download_state()
    assert rel_l2(uu, o.uu, state_floor(o.uu)).max() < 1e-12


@pytest.mark.parametrize("prec", [ffi.PREC_DD, ffi.PREC_FP32], ids=["dd", "fp32"])
@pytest.mark.parametrize("shape", [(512, 8, 16), (16, 8, 512)], ids=["x512", "z512"])
def test_long_lines_incompressible(prec, shape):
    from oracle import laps3d

    kw = dict(if_resis=1, resistivity=2e-4, if_visc=1, viscosity=2e-4, dealias_option=1, cfl=0.4)
    prim = turb(shape, seed=32, kmax=4, rms_u=0.3, rms_b=0.3, p0=1.0)
    o = laps3d.restart3di(shape, kw, prim, 0.0)
    g = ffi.Laps(ffi.params(nx=shape[0], ny=shape[1], nz=shape[2], variant=ffi.VARIANT_3DI, precision=prec, **kw))
    g.upload_state(prim, primitive=True)
    g.set_time(0.0)
    o.dt = 0.0
    for _ in range(2):
        o.step()
    t, dt, status = g.step(2)
    assert status == 0
    uu, _ = g.download_state()
    tol = 1e-11 if prec == ffi.PREC_DD else 1e-5
    assert rel_l2(uu, o.uu, state_floor(o.uu)).max() < tol


@pytest.mark.parametrize("prec", [ffi.PREC_DD, ffi.PREC_FP32], ids=["dd", "fp32"])
def test_2d_1024_rows(prec):
    from oracle import laps3d

    kw = dict(dealias_option=1, cfl=0.4, if_Hall=1, ion_inertial_length=0.05, if_resis=1, resistivity=1e-3,
              if_visc=1, viscosity=1e-3)
    prim = turb((1024, 16, 1), seed=33, kmax=6, rms_u=0.3, rms_b=0.3)
    o = laps3d.restart2d((1024, 16), kw, prim, 0.0)
    g = ffi.Laps(ffi.params(nx=1024, ny=16, nz=1, variant=ffi.VARIANT_2DC, precision=prec, **kw))
    g.upload_state(prim, primitive=True)
    g.set_time(0.0)
    o.dt = 0.0
    for _ in range(3):
        o.step()
    t, dt, status = g.step(3)
    assert status == 0
    uu, _ = g.download_state()
    tol = 1e-11 if prec == ffi.PREC_DD else 1e-5
    assert rel_l2(uu, o.uu, state_floor(o.uu)).max() < tol
