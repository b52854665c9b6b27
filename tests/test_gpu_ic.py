"""laps_init_fields (initial conditions generated on the device) against the oracle.

The state the device generates - background (ifield 0-5), perturbation (ipert 1, 6, 7, 8),
conserved form and forward transform - is downloaded and compared with the oracle's
point-by-point construction of the same fields (oracle/ic.py, which follows
src_compressible/mhdinit.f90:183-1056 and the incompressible variant's ipert 1).  The
random-phase modes are placed in the half spectrum on the device side and summed directly in
the oracle, so agreement also checks the placement (signs, conjugate partners, the kx = 0
plane, modes that meet at one wave vector).  The spectral state must also equal the one an
upload of the oracle's fields gives.
"""
import numpy as np
import pytest

from laps_gb300 import ffi
from laps_gb300.ic import ic_phases
from oracle import ic as oic

pytestmark = pytest.mark.gpu

PI = oic.PI

IC_CASES = {
    "sheet_z": dict(ifield=1, B0=1.0, a0=0.3, T0=0.5),
    "harris_y": dict(ifield=2, U_fast=0.5, U_slow=-0.2, n_fast=1.2, n_slow=0.9, press0=0.8, shear_width=0.1,
                     bx0=0.4, by0=0.1),
    "alfven": dict(ifield=3, ipert=1, bx0=1.0, press0=0.1, db0=0.2, wave_number_jet=2),
    "sheet_y": dict(ifield=4, B0=0.8, a0=0.25, press0=1.0),
    "jet": dict(ifield=5, bx0=1.0, by0=0.2, press0=0.5, Vjet=0.4),
    "waves": dict(ifield=3, ipert=6, bx0=-1.0, press0=1.0, db0=0.05, nmodex=3, nmodey=2, nmodez=3, in_out_ratio=0.7),
    "turb": dict(ifield=3, ipert=7, bx0=1.0, by0=0.2, bz0=-0.1, press0=1.0, db0=0.1, dv0=0.08, drho0=0.02,
                 nmodex=3, nmodey=3, nmodez=2),
    "switchback": dict(ifield=0, ipert=8, rho0=1.0, T0=1.0, B0_SB=1.0, dB_SB=0.4, R0_SB=0.8, R1_SB=0.5, H_SB=0.7,
                       Rm_SB=1.5, Rd_SB=0.4),
}
SHAPE = (16, 16, 32)  # nz, ny, nx


def _oracle(kw, variant, corot=0.0):
    ic = oic.ic_default()
    ic.update(kw)
    ph = ic_phases(ic["ipert"], ic["nmodex"], ic["nmodey"], ic["nmodez"], seed=9)
    u = oic.initial_fields(SHAPE, (2 * PI,) * 3, ic, ph, incompressible=variant == ffi.VARIANT_3DI, cor_angle=corot)
    return ic, ph, u


def _engine(variant, prec, corot=0.0):
    nz, ny, nx = SHAPE
    kw = dict(nx=nx, ny=ny, nz=nz, variant=variant, precision=prec, dealias_option=1)
    if corot:
        kw.update(if_corotating=1, corotating_angle=corot)
    return ffi.Laps(ffi.params(**kw))


def _check(g, u, tol):
    uu, pr = g.download_state()
    got = np.stack([uu[0], pr[0], pr[1], pr[2], uu[4], uu[5], uu[6], pr[3]])
    scale = np.maximum(np.abs(u).max(axis=(1, 2, 3)), 1.0)
    err = (np.abs(got - u).max(axis=(1, 2, 3)) / scale).max()
    assert err < tol, err


@pytest.mark.parametrize("prec", [ffi.PREC_FP64, ffi.PREC_DD, ffi.PREC_FP32], ids=["fp64", "dd", "fp32"])
@pytest.mark.parametrize("case", list(IC_CASES))
def test_init_fields_matches_oracle_3dc(case, prec):
    ic, ph, u = _oracle(IC_CASES[case], ffi.VARIANT_3DC)
    g = _engine(ffi.VARIANT_3DC, prec)
    g.init_fields(ffi.ic_params(**IC_CASES[case]), ph)
    _check(g, u, 1e-12)


@pytest.mark.parametrize("case", ["sheet_z", "harris_y", "alfven", "sheet_y", "waves", "turb", "switchback"])
def test_init_fields_matches_oracle_3di(case):
    ic, ph, u = _oracle(IC_CASES[case], ffi.VARIANT_3DI)
    g = _engine(ffi.VARIANT_3DI, ffi.PREC_FP64)
    g.init_fields(ffi.ic_params(**IC_CASES[case]), ph)
    _check(g, u, 1e-12)


def test_alfven_with_corotation():
    ic, ph, u = _oracle(IC_CASES["alfven"], ffi.VARIANT_3DC, corot=0.4)
    g = _engine(ffi.VARIANT_3DC, ffi.PREC_FP64, corot=0.4)
    g.init_fields(ffi.ic_params(**IC_CASES["alfven"]), ph)
    _check(g, u, 1e-12)


@pytest.mark.parametrize("case", ["turb", "switchback"])
def test_init_fields_equals_upload(case):
    """The generated spectral state is the one laps_upload_state makes of the oracle's fields."""
    ic, ph, u = _oracle(IC_CASES[case], ffi.VARIANT_3DC)
    a = _engine(ffi.VARIANT_3DC, ffi.PREC_FP64)
    a.init_fields(ffi.ic_params(**IC_CASES[case]), ph)
    b = _engine(ffi.VARIANT_3DC, ffi.PREC_FP64)
    b.upload_state(u, primitive=True)
    sa, sb = a.download_spectral(), b.download_spectral()
    assert np.abs(sa - sb).max() <= 1e-13 * np.abs(sb).max()
    # and the two step alike
    for g in (a, b):
        g.set_time(0.0)
    ta = a.step(2)
    tb = b.step(2)
    assert ta[1] == pytest.approx(tb[1], rel=1e-12)
    ua, _ = a.download_state()
    ub, _ = b.download_state()
    assert np.abs(ua - ub).max() <= 1e-11 * np.abs(ub).max()


def test_init_fields_rejects_what_is_not_built():
    g = _engine(ffi.VARIANT_3DC, ffi.PREC_FP64)
    for kw in (dict(ipert=2), dict(ipert=5), dict(ifield=6)):
        with pytest.raises(ffi.LapsError) as e:
            g.init_fields(ffi.ic_params(**kw))
        assert e.value.code == ffi.LAPS_EINVAL
    # phase count and the mode range are checked
    ic = ffi.ic_params(ifield=3, ipert=7, bx0=1.0, nmodex=3, nmodey=3, nmodez=2)
    with pytest.raises(ffi.LapsError):
        g.init_fields(ic, np.zeros(10))
    ic = ffi.ic_params(ifield=3, ipert=7, bx0=1.0, nmodex=3, nmodey=3, nmodez=8)  # nz = 16: |kz| < 8 only
    with pytest.raises(ffi.LapsError):
        g.init_fields(ic, ic_phases(7, 3, 3, 8))
    # ifield 5 exists in the 3-D compressible variant only; the 2-D variant has its own cases
    with pytest.raises(ffi.LapsError):
        _engine(ffi.VARIANT_3DI, ffi.PREC_FP64).init_fields(ffi.ic_params(ifield=5))
    g2 = ffi.Laps(ffi.params(nx=32, ny=32, nz=1, variant=ffi.VARIANT_2DC))
    with pytest.raises(ffi.LapsError):
        g2.init_fields(ffi.ic_params(ifield=3, bx0=1.0, press0=1.0))
