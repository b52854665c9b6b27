"""The initial-condition oracle against the properties the reference's constructions have.

The reference's initial conditions (src_compressible/mhdinit.f90:183-1036) come with no
golden data; each case is built to satisfy an identity, which these tests check on the
oracle's arrays: pressure balance of the current sheets (ifield 1, 4), the Alfven wave's
closed form (ipert 1), divergence-free random-phase fields with the stated mode amplitudes
(ipert 6, 7) and the constant total pressure of the switchback (ipert 8).
"""
import math

import numpy as np
import pytest

from laps_gb300 import ic as gic
from oracle import ic as oic

PI = oic.PI
L3 = (2 * PI, 2 * PI, 2 * PI)


def _ic(**kw):
    d = oic.ic_default()
    d.update(kw)
    return d


def test_alfven_matches_closed_form():
    ic = _ic(ifield=3, ipert=1, bx0=1.0, press0=0.1, db0=0.1)
    u = oic.initial_fields((8, 8, 16), L3, ic, cor_angle=0.3)
    ref = gic.alfven_wave_ic((16, 8, 8), rho0=1.0, p0=0.1, bx0=1.0, db0=0.1, cor_angle=0.3)
    assert np.array_equal(u, ref)


def test_current_sheets_are_in_pressure_balance():
    # ifield 1: rho T0 + Bx^2 / 2 = ninf T0 + B0^2 / 2 (mhdinit.f90:205-222)
    ic = _ic(ifield=1, B0=1.3, a0=0.2, T0=0.7)
    u = oic.background((32, 4, 4), L3, ic)
    ptot = u[7] + 0.5 * u[4] ** 2
    assert np.allclose(ptot, 1.0 * 0.7 + 0.5 * 1.3**2, rtol=0, atol=1e-14)
    # ifield 4: p + Bx^2 / 2 = press0 with uniform density (:258-273)
    ic = _ic(ifield=4, B0=0.8, a0=0.1, press0=2.0)
    u = oic.background((4, 32, 4), L3, ic)
    assert np.allclose(u[7] + 0.5 * u[4] ** 2, 2.0, rtol=0, atol=1e-14)
    assert np.all(u[0] == 1.0)


def _div_spectral(v, L):
    nz, ny, nx = v.shape[1:]
    kx = np.fft.rfftfreq(nx, 1.0 / nx) * 2 * PI / L[0]
    ky = np.fft.fftfreq(ny, 1.0 / ny) * 2 * PI / L[1]
    kz = np.fft.fftfreq(nz, 1.0 / nz) * 2 * PI / L[2]
    f = [np.fft.rfftn(v[c]) for c in range(3)]
    return np.abs(kx[None, None, :] * f[0] + ky[None, :, None] * f[1] + kz[:, None, None] * f[2]).max()


@pytest.mark.parametrize("ipert", [6, 7])
def test_random_phase_fields_are_divergence_free(ipert):
    ic = _ic(ifield=3, ipert=ipert, bx0=1.0, by0=0.3, bz0=-0.2, press0=1.0, db0=0.2, dv0=0.1, drho0=0.05,
             nmodex=3, nmodey=2, nmodez=3, in_out_ratio=0.5)
    ph = gic.ic_phases(ipert, 3, 2, 3, seed=5)
    assert ph.size == oic.nphases(ic)
    u = oic.initial_fields((16, 16, 16), L3, ic, ph)
    bg = oic.background((16, 16, 16), L3, ic)
    du, db = u[1:4] - bg[1:4], u[4:7] - bg[4:7]
    assert np.abs(db).max() > 1e-2
    scale = lambda v: max(np.abs(np.fft.rfftn(v[c])).max() for c in range(3))
    assert _div_spectral(db, L3) < 1e-12 * scale(db)
    assert _div_spectral(du, L3) < 1e-12 * scale(du)


def test_random_phase_mode_amplitudes():
    # ipert 7: |B_hat(k)| = db0 / |k|^{3/2} / 2 per mode (unit-normalised forward transform)
    ic = _ic(ifield=3, ipert=7, bx0=1.0, press0=1.0, db0=0.3, nmodex=2, nmodey=2, nmodez=2)
    ph = gic.ic_phases(7, 2, 2, 2, seed=1)
    u = oic.initial_fields((16, 16, 16), L3, ic, ph)
    b = u[4:7] - np.array([1.0, 0.0, 0.0])[:, None, None, None]
    f = np.stack([np.fft.rfftn(b[c]) / b[0].size for c in range(3)])
    amp = np.sqrt((np.abs(f) ** 2).sum(axis=0))
    for ikx, iky, ikz in [(1, 1, 0), (1, 1, 1), (0, 1, -1), (0, 0, 2), (1, -1, 1)]:
        kr = math.sqrt(ikx**2 + iky**2 + ikz**2)
        k = np.array([ikx, iky, ikz], float)
        perp = np.linalg.norm(np.cross(k, [1.0, 0.0, 0.0])) / np.linalg.norm(k)
        assert amp[ikz % 16, iky % 16, ikx] == pytest.approx(0.3 / kr**1.5 / 2 * perp, rel=1e-12)
    # outside the sphere |k| <= max(nmode) (mhdinit.f90:746-749) and along B0: nothing
    for ikx, iky, ikz in [(2, -1, 0), (2, 2, 2), (1, 0, 0)]:
        assert amp[ikz % 16, iky % 16, ikx] < 1e-15


def test_switchback_keeps_total_pressure():
    ic = _ic(ifield=0, ipert=8, rho0=1.0, T0=1.0, B0_SB=1.0, dB_SB=0.4, R0_SB=0.8, R1_SB=0.5, H_SB=0.7,
             Rm_SB=1.5, Rd_SB=0.4)
    shape = (16, 16, 32)
    u = oic.initial_fields(shape, L3, ic)
    x, y, z = oic.grids(shape, L3)
    r = np.sqrt((y[None, :, None] - PI) ** 2 + (z[:, None, None] - PI) ** 2) + 0 * x[None, None, :]
    ptot = u[7] + 0.5 * (u[4] ** 2 + u[5] ** 2 + u[6] ** 2)
    off = r >= 1e-8
    assert np.allclose(ptot[off], 1.0 + 0.5, rtol=0, atol=1e-13)
    # velocity anti-correlated with B: u = -B / sqrt(rho)
    assert np.allclose(u[1:4], -u[4:7] / np.sqrt(u[0]), rtol=0, atol=1e-15)
    assert np.abs(u[5]).max() > 0.05
