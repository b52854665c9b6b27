"""The FP32-transform modes against the FP64 oracle, through the C-ABI.

LAPS_PREC_FP32 runs the flux transforms and the nonlinear products in FP32 and keeps the
state, the RK register, the CFL arithmetic and the diagnostics in float-float;
LAPS_PREC_FP32_F64 keeps those in IEEE FP64.  Both read and write the state through
transforms of the state's own type, so an upload / download round trip stays at FP64
round-off.  The step error comes from the FP32 right-hand side: a relative error of about
1e-7..1e-6 in RHS, times dt, per stage.

Error bounds (relative L2 per field against the oracle's FP64 run; written here and
reported by bench.py at 256^3):
  upload / download and forward transform     1e-13
  dt from vardt                               1e-5
  one RK stage                                2e-6  (spectrum: 2e-6 of the largest coefficient)
  10 steps                                    1e-5
  100 steps of the 64^3 plain case            2e-5, invariant histories 2e-5
"""
import numpy as np
import pytest

from laps_gb300 import ffi
from oracle.laps3d import forward_3d

from pairs import CONFIG1, CONFIG2, rel_l2, start_pair, state_floor, turb

pytestmark = pytest.mark.gpu

PRECS = [ffi.PREC_FP32, ffi.PREC_FP32_F64]
PREC_ID = ["fp32_dd", "fp32_f64"]


@pytest.mark.parametrize("prec", PRECS, ids=PREC_ID)
def test_state_transforms_stay_at_fp64_roundoff(prec):
    n = (32, 16, 8)
    prim = turb(n, seed=3)
    o, g = start_pair(n, CONFIG1, prim, prec)
    uu, pr = g.download_state()
    assert rel_l2(uu, o.uu, state_floor(o.uu)).max() < 1e-13
    uf = g.download_spectral()
    ref = forward_3d(o.uu)
    assert np.abs(uf - ref).max() / np.abs(ref).max() < 1e-13


@pytest.mark.parametrize("prec", PRECS, ids=PREC_ID)
@pytest.mark.parametrize("case", ["config1", "config2", "corot", "explicit"])
def test_one_stage_error_bound(prec, case):
    n = 32
    kw = {
        "config1": CONFIG1,
        "config2": CONFIG2,
        "corot": dict(CONFIG2, if_corotating=1, corotating_angle=0.3),
        "explicit": dict(CONFIG2, if_resis_exp=1, if_visc_exp=1, if_conserve_background=1),
    }[case]
    prim = turb(n, seed=5, kmax=6, rms_u=0.4, rms_b=0.4)
    o, g = start_pair(n, kw, prim, prec, t0=1.5 if kw.get("if_AEB") else 0.0)
    o.dt = 0.0
    dto = o.vardt()
    dtg = g.vardt()
    assert abs(dtg - dto) <= 1e-5 * dto
    # the stage itself is compared at the same dt: hand the oracle the GPU's dt
    o.dt = dtg
    o.stage(1)
    g.rk_stage(1)
    uu, _ = g.download_state()
    err = rel_l2(uu, o.uu, state_floor(o.uu))
    assert err.max() < 2e-6, err
    uf = g.download_spectral()
    assert np.abs(uf - o.uf).max() <= 2e-6 * np.abs(o.uf).max()


@pytest.mark.parametrize("prec", PRECS, ids=PREC_ID)
@pytest.mark.parametrize("case", ["config1", "config2"])
def test_steps_error_bound(prec, case):
    n = 32
    kw = {"config1": CONFIG1, "config2": CONFIG2}[case]
    prim = turb(n, seed=6, kmax=6, rms_u=0.4, rms_b=0.4)
    o, g = start_pair(n, kw, prim, prec)
    o.dt = 0.0
    nsteps = 10
    for _ in range(nsteps):
        o.vardt()
        o.evolve()
        o.time += o.dt
        o.evolve_radius(o.time)
    t, dt, status = g.step(nsteps)
    assert status == 0
    assert abs(t - o.time) <= 1e-5 * o.time
    uu, _ = g.download_state()
    err = rel_l2(uu, o.uu, state_floor(o.uu))
    assert err.max() < 1e-5, err


@pytest.mark.parametrize("prec", PRECS, ids=PREC_ID)
def test_config1_100_steps_error_bound(prec):
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
    uu, _ = g.download_state()
    err = rel_l2(uu, o.uu, state_floor(o.uu))
    assert err.max() < 2e-5, err
    ho, hg = np.array(hist_o), np.array(hist_g)
    herr = np.abs(hg - ho) / np.maximum(np.abs(ho), 1e-12)
    assert herr.max() < 2e-5, herr


@pytest.mark.parametrize("prec", PRECS, ids=PREC_ID)
@pytest.mark.parametrize("variant", ["3di", "2dc"])
def test_other_variants_error_bound(prec, variant):
    from laps_gb300.ic import turbulence_ic
    from oracle import laps3d

    if variant == "3di":
        kw = dict(if_resis=1, resistivity=5e-4, if_visc=1, viscosity=5e-4, dealias_option=1, cfl=0.4, if_Hall=1,
                  ion_inertial_length=0.05, if_AEB=1, radius0=30.0, Ur0=0.3)
        prim = turbulence_ic(32, seed=12, kmax=5, rms_u=0.4, rms_b=0.4, p0=1.0)
        o = laps3d.restart3di(32, kw, prim, 1.0)
        g = ffi.Laps(ffi.params(nx=32, ny=32, nz=32, variant=ffi.VARIANT_3DI, precision=prec, **kw))
        t0 = 1.0
    else:
        kw = dict(dealias_option=1, cfl=0.4, if_Hall=1, ion_inertial_length=0.05, if_resis=1, resistivity=1e-3,
                  if_visc=1, viscosity=1e-3)
        prim = turbulence_ic((64, 32, 1), seed=13, kmax=6, rms_u=0.4, rms_b=0.4)
        o = laps3d.restart2d((64, 32), kw, prim, 0.0)
        g = ffi.Laps(ffi.params(nx=64, ny=32, nz=1, variant=ffi.VARIANT_2DC, precision=prec, **kw))
        t0 = 0.0
    g.upload_state(prim, primitive=True)
    g.set_time(t0)
    o.dt = 0.0
    for _ in range(5):
        o.step()
    t, dt, status = g.step(5)
    assert status == 0
    uu, _ = g.download_state()
    err = rel_l2(uu, o.uu, state_floor(o.uu))
    assert err.max() < 1e-5, err
