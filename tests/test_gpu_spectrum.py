"""Shell energy spectra on the GPU (laps_spectrum) against the oracle's shell_spectra.

Every shell within 1e-12 of the largest shell (FP64-class state), for the three variants and
the four precision modes right after upload (the FP32-transform modes keep the state and
the spectrum transforms in FP64-class arithmetic); after steps, the FP64 and float-float
runs within 1e-11.  Repeated calls give bitwise-identical shells.
"""
import numpy as np
import pytest

from laps_gb300 import ffi
from laps_gb300.ic import turbulence_ic
from oracle import laps3d

from pairs import CONFIG2, start_pair, turb

pytestmark = pytest.mark.gpu
TWO_PI = 2 * np.pi
ALL = [ffi.PREC_FP64, ffi.PREC_DD, ffi.PREC_FP32, ffi.PREC_FP32_F64]
ALL_ID = ["fp64", "dd", "fp32_dd", "fp32_f64"]


def _close(g, o, tol):
    assert np.abs(g - o).max() <= tol * np.abs(o).max(), np.abs(g - o).max() / np.abs(o).max()


@pytest.mark.parametrize("prec", ALL, ids=ALL_ID)
@pytest.mark.parametrize("n", [16, (32, 16, 8)])
def test_spectrum_after_upload(prec, n):
    prim = turb(n, seed=21, kmax=6)
    o, g = start_pair(n, CONFIG2, prim, prec)
    nshell = 24
    eu, eb = g.spectrum(nshell)
    ou, ob = laps3d.shell_spectra(o.uu, TWO_PI, TWO_PI, TWO_PI, nshell)
    _close(eu, ou, 1e-12)
    _close(eb, ob, 1e-12)
    eu2, eb2 = g.spectrum(nshell)
    assert np.array_equal(eu, eu2) and np.array_equal(eb, eb2)


@pytest.mark.parametrize("prec", [ffi.PREC_FP64, ffi.PREC_DD], ids=["fp64", "dd"])
def test_spectrum_after_steps(prec):
    n = 32
    prim = turb(n, seed=22, kmax=6, rms_u=0.4, rms_b=0.4)
    o, g = start_pair(n, CONFIG2, prim, prec)
    o.dt = 0.0
    for _ in range(5):
        o.vardt(); o.evolve(); o.time += o.dt; o.evolve_radius(o.time)
    g.step(5)
    eu, eb = g.spectrum(40)
    ou, ob = laps3d.shell_spectra(o.uu, TWO_PI, TWO_PI, TWO_PI, 40)
    _close(eu, ou, 1e-11)
    _close(eb, ob, 1e-11)
    # the 2/3 sphere leaves B nothing beyond |k| = n/3 (u = rho u / rho is not band-limited)
    assert eb[12:].max() < 1e-20 * eb.max()


@pytest.mark.parametrize("prec", [ffi.PREC_FP64, ffi.PREC_DD], ids=["fp64", "dd"])
def test_spectrum_2d_and_incompressible(prec):
    kw2 = dict(dealias_option=1, cfl=0.4, if_Hall=1, ion_inertial_length=0.05)
    prim = turbulence_ic((64, 32, 1), seed=23, kmax=6, rms_u=0.3, rms_b=0.3)
    g = ffi.Laps(ffi.params(nx=64, ny=32, nz=1, variant=ffi.VARIANT_2DC, precision=prec, Lx=TWO_PI, Ly=TWO_PI / 2, **kw2))
    g.upload_state(prim, primitive=True)
    o = laps3d.restart2d((64, 32), dict(kw2, Lx=TWO_PI, Ly=TWO_PI / 2), prim, 0.0)
    eu, eb = g.spectrum(50)
    ou, ob = laps3d.shell_spectra(o.uu, TWO_PI, TWO_PI / 2, 1.0, 50)
    _close(eu, ou, 1e-12)
    _close(eb, ob, 1e-12)
    kwi = dict(dealias_option=1, cfl=0.4)
    prim = turbulence_ic(16, seed=24, kmax=5, p0=1.0)
    g = ffi.Laps(ffi.params(nx=16, ny=16, nz=16, variant=ffi.VARIANT_3DI, precision=prec, **kwi))
    g.upload_state(prim, primitive=True)
    o = laps3d.restart3di(16, kwi, prim, 0.0)
    eu, eb = g.spectrum(16)
    ou, ob = laps3d.shell_spectra(o.uu, TWO_PI, TWO_PI, TWO_PI, 16)
    _close(eu, ou, 1e-12)
    _close(eb, ob, 1e-12)


def test_spectrum_rejects_bad_shell_count():
    prim = turb(16, seed=25)
    g = ffi.Laps(ffi.params(nx=16, ny=16, nz=16, precision=ffi.PREC_FP64))
    g.upload_state(prim, primitive=True)
    with pytest.raises(ffi.LapsError):
        g.spectrum(0)
