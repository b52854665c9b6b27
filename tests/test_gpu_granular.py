"""The granular entry points against the oracle's subroutines one by one: calc_flux,
transform_flux_real_to_fourier, calc_rhs (mhdrhs.f90) and dealias (dealiasing.f90), for the
3-D Hall + expanding-box case and a 2-D case, FP64 and float-float: every field within 1e-12
of its largest value; the state is left unchanged by calc_rhs."""
import numpy as np
import pytest

from laps_gb300 import ffi
from laps_gb300.ic import turbulence_ic
from oracle import laps3d

from pairs import CONFIG2, start_pair, turb

pytestmark = pytest.mark.gpu
PRECS = [ffi.PREC_FP64, ffi.PREC_DD]
PREC_ID = ["fp64", "dd"]


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _pair(case, prec):
    if case == "3dc":
        n = (32, 16, 16)
        prim = turb(n, seed=51, kmax=5, rms_u=0.4, rms_b=0.4)
        return start_pair(n, CONFIG2, prim, prec, t0=1.5)
    kw = dict(dealias_option=1, cfl=0.4, if_Hall=1, ion_inertial_length=0.05, if_AEB=1, radius0=30.0, Ur0=0.3)
    prim = turbulence_ic((64, 32, 1), seed=52, kmax=6, rms_u=0.3, rms_b=0.3)
    o = laps3d.restart2d((64, 32), kw, prim, 1.0)
    g = ffi.Laps(ffi.params(nx=64, ny=32, nz=1, variant=ffi.VARIANT_2DC, precision=prec, **kw))
    g.upload_state(prim, primitive=True)
    g.set_time(1.0)
    return o, g


@pytest.mark.parametrize("prec", PRECS, ids=PREC_ID)
@pytest.mark.parametrize("case", ["3dc", "2dc"])
def test_flux_transform_rhs_match_oracle(prec, case):
    o, g = _pair(case, prec)
    flux, expand = o.calc_flux()
    fg = g.calc_flux()
    nf = 18 + (1 if expand is not None else 0)
    assert fg.shape[0] == nf
    for k in range(18):
        assert _rel(fg[k], flux[k]) < 1e-12, k
    if expand is not None:
        assert _rel(fg[18], expand) < 1e-12
    ff, ef = o.transform_flux_real_to_fourier(flux, expand)
    tg = g.transform_flux()
    for k in range(18):
        assert np.abs(tg[k] - ff[k]).max() <= 1e-12 * np.abs(ff).max(), k
    if ef is not None:
        assert np.abs(tg[18] - ef).max() <= 1e-12 * np.abs(ef).max()
    before = g.download_spectral()
    fnl = o.calc_rhs(ff, ef)
    rg = g.calc_rhs()
    assert np.abs(rg - fnl).max() <= 1e-12 * np.abs(fnl).max()
    assert np.array_equal(g.download_spectral(), before)  # the state is untouched
    # a step after calc_rhs is the step without it
    t, dt, st = g.step(2)
    h = _pair(case, prec)[1]
    t2, dt2, st2 = h.step(2)
    assert st == 0 and t == t2 and np.array_equal(g.download_spectral(), h.download_spectral())


@pytest.mark.parametrize("prec", PRECS, ids=PREC_ID)
@pytest.mark.parametrize("option", [1, 2])
def test_dealias_matches_oracle(prec, option):
    n = 32
    kw = dict(CONFIG2, dealias_option=option)
    prim = turb(n, seed=53, kmin=1, kmax=15, rms_u=0.3, rms_b=0.3)  # content beyond the 2/3 sphere
    o, g = start_pair(n, kw, prim, prec)
    g.dealias()
    o.dealias()
    uf = g.download_spectral()
    assert np.abs(uf - o.uf).max() <= 1e-13 * np.abs(o.uf).max()


def test_incompressible_flux_calls_rejected():
    g = ffi.Laps(ffi.params(nx=16, ny=16, nz=16, variant=ffi.VARIANT_3DI))
    g.upload_state(turbulence_ic(16, seed=54, p0=1.0), primitive=True)
    with pytest.raises(ffi.LapsError):
        g.calc_rhs()
