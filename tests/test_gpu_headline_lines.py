"""GPU parity at the line lengths of the measured workloads: 128- and 256-point lines.

The 256^3 Hall + expanding-box benchmark runs the 256-point instances of every pass (the
float-float 256-point x rows use the shared, non-inlined row transform), and the 2-D
ensemble's 128^2 and 256^2 members run the 128- and 256-point instances.  Each of them is
checked here against the oracle (the CPU restatement of the reference), through the C-ABI:

  * 3-D compressible Hall + expanding box on grids with one 128- or 256-point axis, in all
    four arithmetic modes, for one RK stage and for 10 steps;
  * the 3-D incompressible variant with a 256-point axis;
  * 2-D members at 128^2 and 256^2;
  * the full 256^3 benchmark case for 2 steps.

Tolerances (relative L2 per field, written per test): FP64 and float-float one stage
1e-12, steps 1e-11; the FP32-transform modes carry the FP32 right-hand side's error,
one stage 2e-6 and steps 1e-5 (the bounds of tests/test_gpu_fp32.py).
"""
import numpy as np
import pytest

from laps_gb300 import ffi
from laps_gb300.ic import turbulence_ic
from oracle import laps3d

from pairs import CONFIG2, rel_l2, start_pair, state_floor, turb

pytestmark = pytest.mark.gpu

PRECS = [ffi.PREC_FP64, ffi.PREC_DD, ffi.PREC_FP32, ffi.PREC_FP32_F64]
PREC_ID = ["fp64", "dd", "fp32_dd", "fp32_f64"]
SHAPES = [(256, 16, 8), (16, 256, 8), (16, 8, 256), (128, 16, 8), (16, 128, 8), (16, 8, 128)]
SHAPE_ID = ["x256", "y256", "z256", "x128", "y128", "z128"]


def _tols(prec):
    """(one stage, steps, dt) bounds of the mode."""
    if prec in (ffi.PREC_FP64, ffi.PREC_DD):
        return 1e-12, 1e-11, 1e-13
    return 2e-6, 1e-5, 1e-5


@pytest.mark.parametrize("prec", PRECS, ids=PREC_ID)
@pytest.mark.parametrize("shape", SHAPES, ids=SHAPE_ID)
def test_one_stage(prec, shape):
    tol_stage, _, tol_dt = _tols(prec)
    prim = turb(shape, seed=41, kmax=3, rms_u=0.4, rms_b=0.4)
    o, g = start_pair(shape, CONFIG2, prim, prec, t0=1.5)
    o.dt = 0.0
    dto = o.vardt()
    dtg = g.vardt()
    assert abs(dtg - dto) <= tol_dt * dto
    o.dt = dtg  # the stage itself at the same dt
    o.stage(1)
    g.rk_stage(1)
    uu, _ = g.download_state()
    err = rel_l2(uu, o.uu, state_floor(o.uu))
    assert err.max() < tol_stage, err
    uf = g.download_spectral()
    assert np.abs(uf - o.uf).max() <= tol_stage * np.abs(o.uf).max()


@pytest.mark.parametrize("prec", PRECS, ids=PREC_ID)
@pytest.mark.parametrize("shape", SHAPES, ids=SHAPE_ID)
def test_ten_steps(prec, shape):
    _, tol_steps, tol_dt = _tols(prec)
    prim = turb(shape, seed=42, kmax=3, rms_u=0.4, rms_b=0.4)
    o, g = start_pair(shape, CONFIG2, prim, prec)
    o.dt = 0.0
    for _ in range(10):
        o.vardt(); o.evolve(); o.time += o.dt; o.evolve_radius(o.time)
    t, dt, status = g.step(10)
    assert status == 0
    assert abs(t - o.time) <= tol_dt * o.time
    uu, _ = g.download_state()
    err = rel_l2(uu, o.uu, state_floor(o.uu))
    assert err.max() < tol_steps, err


@pytest.mark.parametrize("prec", PRECS, ids=PREC_ID)
def test_incompressible_x256(prec):
    _, tol_steps, _ = _tols(prec)
    shape = (256, 16, 8)
    kw = dict(if_resis=1, resistivity=2e-4, if_visc=1, viscosity=2e-4, dealias_option=1, cfl=0.4, if_Hall=1,
              ion_inertial_length=0.05)
    prim = turb(shape, seed=43, kmax=3, rms_u=0.3, rms_b=0.3, p0=1.0)
    o = laps3d.restart3di(shape, kw, prim, 0.0)
    g = ffi.Laps(ffi.params(nx=shape[0], ny=shape[1], nz=shape[2], variant=ffi.VARIANT_3DI, precision=prec, **kw))
    g.upload_state(prim, primitive=True)
    g.set_time(0.0)
    o.dt = 0.0
    for _ in range(3):
        o.step()
    t, dt, status = g.step(3)
    assert status == 0
    uu, _ = g.download_state()
    assert rel_l2(uu, o.uu, state_floor(o.uu)).max() < tol_steps


@pytest.mark.parametrize("prec", PRECS, ids=PREC_ID)
@pytest.mark.parametrize("n", [128, 256])
def test_2d_member(prec, n):
    """An ensemble member's grid: 2-D Hall-MHD at n^2 with 3 steps."""
    _, tol_steps, tol_dt = _tols(prec)
    kw = dict(dealias_option=1, cfl=0.4, if_Hall=1, ion_inertial_length=0.05, if_resis=1, resistivity=1e-3,
              if_visc=1, viscosity=1e-3)
    prim = turbulence_ic((n, n, 1), seed=44, kmax=8, rms_u=0.3, rms_b=0.3)
    o = laps3d.restart2d((n, n), kw, prim, 0.0)
    g = ffi.Laps(ffi.params(nx=n, ny=n, nz=1, variant=ffi.VARIANT_2DC, precision=prec, **kw))
    g.upload_state(prim, primitive=True)
    g.set_time(0.0)
    o.dt = 0.0
    for _ in range(3):
        o.step()
    t, dt, status = g.step(3)
    assert status == 0
    assert abs(dt - o.dt) <= tol_dt * o.dt
    uu, _ = g.download_state()
    assert rel_l2(uu, o.uu, state_floor(o.uu)).max() < tol_steps


@pytest.fixture(scope="module")
def bench_case_oracle():
    """The 256^3 benchmark case (Hall d_i = 0.05, Ur0/R0 = 0.01, eta = nu = 5e-4, random-phase
    1 <= |k| <= 8 spectrum with rms 0.5, seed 1) advanced 2 steps by the oracle."""
    n = 256
    prim = turbulence_ic(n, kmin=1, kmax=8, alpha=-1.0, rms_u=0.5, rms_b=0.5, seed=1)
    o = laps3d.restart(n, CONFIG2, prim)
    o.dt = 0.0
    dts = []
    for _ in range(2):
        o.vardt(); o.evolve(); o.time += o.dt; o.evolve_radius(o.time)
        dts.append(o.dt)
    return prim, o.uu.copy(), o.time, dts


@pytest.mark.parametrize("prec", PRECS, ids=PREC_ID)
def test_bench_case_256_cubed_two_steps(prec, bench_case_oracle):
    """The full benchmark grid: every 256-point pass instance, pruned geometry and CFL
    screen at the measured size, against the oracle after 2 steps (FP64 / float-float
    1e-12; FP32-transform modes 1e-5)."""
    prim, uu_o, t_o, dts = bench_case_oracle
    tol = 1e-12 if prec in (ffi.PREC_FP64, ffi.PREC_DD) else 1e-5
    tol_dt = 1e-13 if prec in (ffi.PREC_FP64, ffi.PREC_DD) else 1e-5
    g = ffi.Laps(ffi.params(nx=256, ny=256, nz=256, precision=prec, **CONFIG2))
    g.upload_state(prim, primitive=True)
    g.set_time(0.0)
    t, dt, status = g.step(2)
    assert status == 0
    assert abs(dt - dts[-1]) <= tol_dt * dts[-1]
    assert abs(t - t_o) <= tol_dt * t_o
    uu, _ = g.download_state()
    g.close()
    err = rel_l2(uu, uu_o, state_floor(uu_o))
    assert err.max() < tol, err
