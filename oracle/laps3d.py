"""CPU restatement (oracle) of LAPS's 3D compressible RHS evaluation and RK3 time advance.

TEST INFRASTRUCTURE ONLY.  Nothing in the shipped GPU path imports this module; it is
imported only by ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py``, always as the oracle, never as the thing measured or shipped.

PARITY UNPINNED.  The reference (Fortran 90 + MPI + FFTW3, ``src_compressible/``) cannot
be compiled here (no Fortran compiler, no MPI, no FFTW) and ships no tests, golden vectors
or fixtures.  This file restates its algorithm line by line (citations below are
``file:line`` inside the reference project); it is anchored by analytic known-answer tests
built from the reference's own initial conditions (the ``ipert=1`` circularly polarised
Alfven wave, ``src_compressible/mhdinit.f90:328-342``) and by conservation properties,
not by outputs of the reference binary.

Array conventions (identical memory order to the reference's Fortran arrays):
  real-space field   ``uu[ivar, iz, iy, ix]``       == Fortran ``uu(ix,iy,iz,ivar)``
  spectral field     ``uf[ivar, kz, ky, kx]``       == Fortran ``uu_fourier(kx,ky,kz,ivar)``
with ``kx`` in ``0..nx/2`` (half spectrum) and ``ky``, ``kz`` in FFT order.

Third-party arithmetic: the reference's FFTs are FFTW3 1-D plans (``FFTW_ESTIMATE``,
version not pinned; ``src_compressible/makefile:6-13``).  They compute the unnormalised
DFT ``X_k = sum_j x_j exp(-+2 pi i jk/n)``; the c2r transform ignores the imaginary parts of
the DC and Nyquist inputs.  ``numpy.fft`` / ``scipy.fft`` (pocketfft) compute the same
transforms; results agree to round-off.
"""
from __future__ import annotations

import dataclasses
import math
import os

import numpy as np

try:  # pocketfft with threads when scipy is present (same transforms as numpy.fft)
    import scipy.fft as _sfft

    _WORKERS = int(os.environ.get("LAPS_ORACLE_THREADS", "0")) or os.cpu_count() or 1

    def _fft(a, axis):
        return _sfft.fft(a, axis=axis, workers=_WORKERS)

    def _ifft_unnorm(a, axis):
        return _sfft.ifft(a, axis=axis, norm="forward", workers=_WORKERS)

    def _rfft(a, axis):
        return _sfft.rfft(a, axis=axis, workers=_WORKERS)

    def _irfft_unnorm(a, n, axis):
        return _sfft.irfft(a, n=n, axis=axis, norm="forward", workers=_WORKERS)

except ImportError:  # pragma: no cover - numpy fallback
    def _fft(a, axis):
        return np.fft.fft(a, axis=axis)

    def _ifft_unnorm(a, axis):
        return np.fft.ifft(a, axis=axis, norm="forward")

    def _rfft(a, axis):
        return np.fft.rfft(a, axis=axis)

    def _irfft_unnorm(a, n, axis):
        return np.fft.irfft(a, n=n, axis=axis, norm="forward")


PI = 3.141592653589793  # src_compressible/mhdinit.f90:7 (``real :: pi``, -r8)

# variable slots, src_compressible/mhdinit.f90:30-33
RHO, MX, MY, MZ, BX, BY, BZ, EN = range(8)


@dataclasses.dataclass
class Params3D:
    """Namelist values the hot path reads (``src_compressible/mhd.f90:30-41``).

    Defaults are the reference's module initialisers: ``mhdinit.f90:21-26``,
    ``dealiasing.f90:10-12``, ``mhd.f90:21`` (cfl), ``AEBmod.f90:10-12``.
    """

    nx: int = 32
    ny: int = 32
    nz: int = 32
    Lx: float = 2 * PI
    Ly: float = 2 * PI
    Lz: float = 2 * PI
    adiabatic_index: float = 5.0 / 3.0
    if_resis: bool = False
    resistivity: float = 0.0
    if_resis_exp: bool = False
    if_visc: bool = False
    viscosity: float = 0.0
    if_visc_exp: bool = False
    if_conserve_background: bool = False
    dealias_option: int = 2
    afx: float = 0.495
    afy: float = 0.495
    afz: float = 0.495
    cfl: float = 0.5
    if_AEB: bool = False
    radius0: float = 30.0
    Ur0: float = 0.0
    if_corotating: bool = False
    corotating_angle: float = 0.0
    if_Hall: bool = False
    ion_inertial_length: float = 0.0


def wave_numbers(n: int, L: float) -> np.ndarray:
    """k_i = 2 pi (i-1)/L for i <= n/2+1, else 2 pi (i-1-n)/L; the Nyquist index takes +k.

    ``src_compressible/mhdinit.f90:88-115``.
    """
    i = np.arange(n, dtype=np.float64)
    return np.where(np.arange(n) <= n // 2, (2 * PI * i) / L, (2 * PI * (i - n)) / L)


# ----------------------------------------------------------------------------- transforms
def forward_3d(u: np.ndarray) -> np.ndarray:
    """Real -> half spectrum; each axis divided by its length after its pass.

    x r2c / nx (``fftw.f90:60-62``), y c2c / ny (``fftw.f90:156-161``), z c2c / nz
    (``fftw.f90:173-178``).  Works on ``[..., z, y, x]``.
    """
    nz, ny, nx = u.shape[-3:]
    w = _rfft(u, axis=-1) / nx
    w = _fft(w, axis=-2) / ny
    w = _fft(w, axis=-3) / nz
    return w


def inverse_3d(w: np.ndarray, nx: int) -> np.ndarray:
    """Half spectrum -> real, unnormalised: z c2c, y c2c, x c2r (``fftw.f90:182-222,94-99``)."""
    v = _ifft_unnorm(w, axis=-3)
    v = _ifft_unnorm(v, axis=-2)
    return _irfft_unnorm(v, nx, axis=-1)


# ----------------------------------------------------------------------------- the solver
class Laps3DC:
    """State and routines of the 3-D compressible solver, one method per reference routine."""

    def __init__(self, p: Params3D):
        self.p = p
        nx, ny, nz = p.nx, p.ny, p.nz
        self.dx, self.dy, self.dz = p.Lx / nx, p.Ly / ny, p.Lz / nz
        self.wx = wave_numbers(nx, p.Lx)[: nx // 2 + 1]
        self.wy = wave_numbers(ny, p.Ly)
        self.wz = wave_numbers(nz, p.Lz)
        # AEB_initialize: with the expanding box off, Ur0 is forced to 0 (mhd.f90:88-90)
        self.Ur0 = p.Ur0 if p.if_AEB else 0.0
        ang = p.corotating_angle if p.if_corotating else 0.0  # AEBmod.f90:28-30
        self.cos_cor = math.cos(ang)
        self.sin_cor = math.sin(ang)
        self.radius = p.radius0
        self.tau_exp = self._tau(self.radius)
        # grid_initialize k^2 (mhdinit.f90:117-123): plain sum, no radius factor
        self.k_square = (self.wx[None, None, :] ** 2 + self.wy[None, :, None] ** 2) + self.wz[:, None, None] ** 2
        self._init_dealias()
        self.uu = None
        self.uu_prim = None
        self.uf = None
        self.fnl_rk = np.zeros((8, nz, ny, nx // 2 + 1), np.complex128)
        self.cc1 = np.zeros(3)
        self.dd1 = np.zeros(3)
        self.time_step = np.zeros(3)
        self.dt = 0.0
        self.time = 0.0

    # ------------------------------------------------------------------ AEBmod.f90
    def _tau(self, r):
        """tau_exp = R / Ur (``AEBmod.f90:46-54``); +inf when Ur = 0 (unused then)."""
        with np.errstate(divide="ignore"):
            return np.float64(r) / np.float64(self.Ur0) if self.Ur0 != 0.0 else math.inf

    def evolve_radius(self, t):
        """R = R0 + Ur t, tau = R/Ur, then update_ksquare (``AEBmod.f90:56-73,87-125``)."""
        p = self.p
        self.radius = p.radius0 + self.Ur0 * t
        self.tau_exp = self._tau(self.radius)
        kx = self.wx[None, None, :]
        ky = self.wy[None, :, None]
        kz = self.wz[:, None, None]
        R0, R = p.radius0, self.radius
        if p.if_corotating:
            c, s = self.cos_cor, self.sin_cor
            self.k_square = (
                kx**2 * (c**2 + (s * R0 / R) ** 2)
                + ky**2 * (s**2 + (c * R0 / R) ** 2)
                + kx * ky * 2 * c * s * (1 - (R0 / R) ** 2)
                + (kz * R0 / R) ** 2
            )
        else:
            self.k_square = kx**2 + (ky * R0 / R) ** 2 + (kz * R0 / R) ** 2

    def ik(self):
        """The derivative factors (i kx, i ky, i kz) as real magnitudes a with d/dx -> i a.

        ``mhdrhs.f90:191-204``: ky, kz scaled by R0/R; corotation mixes kx and ky.
        """
        p = self.p
        R0, R = p.radius0, self.radius
        kx = np.broadcast_to(self.wx[None, None, :], self.k_square.shape)
        ky = np.broadcast_to((self.wy * R0 / R)[None, :, None], self.k_square.shape)
        kz = np.broadcast_to((self.wz * R0 / R)[:, None, None], self.k_square.shape)
        if p.if_AEB and p.if_corotating:
            wx = self.wx[None, None, :]
            wy = self.wy[None, :, None]
            kx = np.broadcast_to(wx * self.cos_cor + wy * self.sin_cor, self.k_square.shape)
            ky = np.broadcast_to((-wx * self.sin_cor + wy * self.cos_cor) * R0 / R, self.k_square.shape)
        return kx, ky, kz

    # ------------------------------------------------------------------ dealiasing.f90
    def _init_dealias(self):
        """Option 1: spherical mask of normalised radius 1/3; option 2: compact filter.

        ``dealiasing.f90:8,13-67``.
        """
        p = self.p
        if p.dealias_option == 1:
            rx = (self.wx * p.Lx / (2 * PI * p.nx)) ** 2
            ry = (self.wy * p.Ly / (2 * PI * p.ny)) ** 2
            rz = (self.wz * p.Lz / (2 * PI * p.nz)) ** 2
            rad = np.sqrt((rx[None, None, :] + ry[None, :, None]) + rz[:, None, None])
            self.keep = ~(rad > 1.0 / 3.0)
        elif p.dealias_option == 2:
            def filt(w, L, n, af):
                aj = (5.0 + 6.0 * af) / 8.0
                bj = (1.0 + 2.0 * af) / 2.0
                cj = -(1.0 - 2 * af) / 8.0
                wl = w * L / n
                return (aj + bj * np.cos(wl) + cj * np.cos(2 * wl)) / (1 + 2 * af * np.cos(wl))

            self.filtx = filt(self.wx, p.Lx, p.nx, p.afx)
            self.filty = filt(self.wy, p.Ly, p.ny, p.afy)
            self.filtz = filt(self.wz, p.Lz, p.nz, p.afz)

    def dealias(self):
        """``dealiasing.f90:70-113``."""
        p = self.p
        if p.dealias_option == 1:
            self.uf[:, ~self.keep] = 0.0
        elif p.dealias_option == 2:
            self.uf = ((self.uf * self.filtx[None, None, None, :]) * self.filty[None, None, :, None]) * self.filtz[
                None, :, None, None
            ]

    # ------------------------------------------------------------------ init / state
    def initial_calc_conserve_variable(self, prim: np.ndarray):
        """Primitive (rho, u, B, p) -> conserved (rho, rho u, B, e); ``mhdinit.f90:1038-1056``."""
        g = self.p.adiabatic_index
        uu = np.array(prim, dtype=np.float64, copy=True)
        self.uu_prim = np.empty((4,) + uu.shape[1:])
        self.uu_prim[0:3] = uu[1:4]
        self.uu_prim[3] = uu[7]
        uu[1] = uu[0] * self.uu_prim[0]
        uu[2] = uu[0] * self.uu_prim[1]
        uu[3] = uu[0] * self.uu_prim[2]
        uu[7] = self.uu_prim[3] / (g - 1) + 0.5 * (
            uu[0] * (self.uu_prim[0] ** 2 + self.uu_prim[1] ** 2 + self.uu_prim[2] ** 2)
            + uu[4] ** 2 + uu[5] ** 2 + uu[6] ** 2
        )
        self.uu = uu

    def set_conserved(self, uu: np.ndarray):
        """Load a conserved state and recompute the primitives from it."""
        self.uu = np.array(uu, dtype=np.float64, copy=True)
        self.update_uu_prim_from_uu()

    def transform_uu_real_to_fourier(self):
        """``fftw.f90:42-71``."""
        self.uf = forward_3d(self.uu)

    def transform_uu_fourier_to_real(self):
        """``fftw.f90:73-103``."""
        self.uu = inverse_3d(self.uf, self.p.nx)

    def update_uu_prim_from_uu(self):
        """u = rho u / rho; p = (e - (rho u . u + B^2)/2)(gamma - 1); ``mhdrhs.f90:282-294``."""
        uu = self.uu
        g = self.p.adiabatic_index
        prim = np.empty((4,) + uu.shape[1:])
        prim[0] = uu[1] / uu[0]
        prim[1] = uu[2] / uu[0]
        prim[2] = uu[3] / uu[0]
        prim[3] = (uu[7] - 0.5 * (uu[1] * prim[0] + uu[2] * prim[1] + uu[3] * prim[2]
                                  + uu[4] ** 2 + uu[5] ** 2 + uu[6] ** 2)) * (g - 1)
        self.uu_prim = prim

    # ------------------------------------------------------------------ mhdrhs.f90
    def calc_current_density_real(self):
        """J = ik x B in spectral space, then 3 inverse transforms; ``mhdrhs.f90:296-362``."""
        kx, ky, kz = self.ik()
        uf = self.uf
        i = 1j
        jf = np.stack([
            i * ky * uf[BZ] - i * kz * uf[BY],
            i * kz * uf[BX] - i * kx * uf[BZ],
            i * kx * uf[BY] - i * ky * uf[BX],
        ])
        return inverse_3d(jf, self.p.nx)

    def calc_flux(self):
        """The 18 real-space fluxes (+ the expansion energy term); ``mhdrhs.f90:21-124``.

        Order: rho u (1:3), momentum rows Txx,Tyx,Tzx / Txy,Tyy,Tzy / Txz,Tyz,Tzz (4:12),
        E = -u x B (+ Hall) (13:15), energy flux (16:18); returns (flux[18], expand or None).
        """
        p = self.p
        uu, pr = self.uu, self.uu_prim
        g = p.adiabatic_index
        P = pr[3]
        Bx, By, Bz = uu[BX], uu[BY], uu[BZ]
        ux, uy, uz = pr[0], pr[1], pr[2]
        rho = uu[RHO]
        ptot = P + 0.5 * (Bx**2 + By**2 + Bz**2)
        udotb = ux * Bx + uy * By + uz * Bz
        f = np.empty((18,) + uu.shape[1:])
        f[0:3] = uu[1:4]
        f[3] = uu[MX] * ux - Bx * Bx + ptot
        f[4] = uu[MY] * ux - By * Bx
        f[5] = uu[MZ] * ux - Bz * Bx
        f[6] = uu[MX] * uy - Bx * By
        f[7] = uu[MY] * uy - By * By + ptot
        f[8] = uu[MZ] * uy - Bz * By
        f[9] = uu[MX] * uz - Bx * Bz
        f[10] = uu[MY] * uz - By * Bz
        f[11] = uu[MZ] * uz - Bz * Bz + ptot
        f[12] = uz * By - uy * Bz
        f[13] = ux * Bz - uz * Bx
        f[14] = uy * Bx - ux * By
        f[15] = (uu[EN] + ptot) * ux - udotb * Bx
        f[16] = (uu[EN] + ptot) * uy - udotb * By
        f[17] = (uu[EN] + ptot) * uz - udotb * Bz
        expand = None
        if p.if_AEB:
            expand = self.expand_term(P, Bx, By, Bz, uu, ux, uy, uz, g, self.tau_exp)
        if p.if_Hall:
            J = self.calc_current_density_real()
            di = p.ion_inertial_length
            f[12] = f[12] + di / rho * (J[1] * uu[BZ] - J[2] * uu[BY])
            f[13] = f[13] + di / rho * (J[2] * uu[BX] - J[0] * uu[BZ])
            f[14] = f[14] + di / rho * (J[0] * uu[BY] - J[1] * uu[BX])
        return f, expand

    def expand_term(self, P, Bx, By, Bz, uu, ux, uy, uz, g, tau):
        """Energy source of the expanding box (``mhdrhs.f90:93-103``)."""
        return (-2 * g / (g - 1) * P / tau
                - (2.0 * Bx**2 + By**2 + Bz**2) / tau
                - (uu[MX] * ux + 2 * uu[MY] * uy + 2 * uu[MZ] * uz) / tau)

    def expansion_coefficients(self):
        """Damping factors of rho, rho u, B in calc_rhs (``mhdrhs.f90:235-247``)."""
        return (2.0, 2.0, 3.0, 3.0, 2.0, 1.0, 1.0)

    def transform_flux_real_to_fourier(self, flux, expand):
        """``mhdrhs.f90:128-172``."""
        ff = forward_3d(flux)
        ef = forward_3d(expand) if expand is not None else None
        return ff, ef

    def calc_rhs(self, ff, ef):
        """fnl = -ik.F, curl E, expansion damping, explicit diffusion; ``mhdrhs.f90:174-279``."""
        p = self.p
        kx, ky, kz = self.ik()
        i = 1j
        uf = self.uf
        fnl = np.empty_like(uf)
        fnl[0] = -(i * kx * ff[0] + i * ky * ff[1] + i * kz * ff[2])
        fnl[1] = -(i * kx * ff[3] + i * ky * ff[4] + i * kz * ff[5])
        fnl[2] = -(i * kx * ff[6] + i * ky * ff[7] + i * kz * ff[8])
        fnl[3] = -(i * kx * ff[9] + i * ky * ff[10] + i * kz * ff[11])
        fnl[4] = i * kz * ff[13] - i * ky * ff[14]
        fnl[5] = i * kx * ff[14] - i * kz * ff[12]
        fnl[6] = i * ky * ff[12] - i * kx * ff[13]
        fnl[7] = -(i * kx * ff[15] + i * ky * ff[16] + i * kz * ff[17])
        if p.if_AEB:
            tau = self.tau_exp
            for v, c in enumerate(self.expansion_coefficients()):
                fnl[v] = fnl[v] - c * uf[v] / tau
            fnl[7] = fnl[7] + ef
        if p.if_visc and p.if_visc_exp:
            for v in (1, 2, 3):
                fnl[v] = fnl[v] - p.viscosity * uf[v] * self.k_square
        if p.if_resis and p.if_resis_exp:
            ks = self.k_square
            m = np.ones(ks.shape, bool)
            if p.if_conserve_background:
                m[0, :, 0] = False  # (ix == 1) .and. (iz == 1) is skipped
            for v in (4, 5, 6):
                fnl[v] = np.where(m, fnl[v] - p.resistivity * uf[v] * ks, fnl[v])
        return fnl

    # ------------------------------------------------------------------ rktmod.f90
    def rkt_init(self, dt):
        """Low-storage RK3 coefficients, zero fnl_rk; ``rktmod.f90:15-32``."""
        self.fnl_rk[...] = 0.0
        self.cc1[:] = (8.0 / 15.0 * dt, 5.0 / 12.0 * dt, 0.75 * dt)
        self.dd1[:] = (0.0, -17.0 / 60.0 * dt, -5.0 / 12.0 * dt)
        self.time_step[:] = (8.0 / 15.0 * dt, 2.0 / 15.0 * dt, 1.0 / 3.0 * dt)

    def rkt(self, irk, fnl):
        """uu_f = cc fnl + dd fnl_rk + uu_f, then implicit nu/eta; ``rktmod.f90:34-62``. irk is 1-based."""
        p = self.p
        k = irk - 1
        self.uf = self.cc1[k] * fnl + self.dd1[k] * self.fnl_rk + self.uf
        self.fnl_rk = fnl.copy()
        if p.if_visc and not p.if_visc_exp:
            d = self.time_step[k] * self.k_square * p.viscosity + 1.0
            for v in (1, 2, 3):
                self.uf[v] = self.uf[v] / d
        if p.if_resis and not p.if_resis_exp:
            d = self.time_step[k] * self.k_square * p.resistivity + 1.0
            for v in (4, 5, 6):
                self.uf[v] = self.uf[v] / d

    # ------------------------------------------------------------------ mhd.f90
    def stage(self, irk):
        """One RK stage of ``evolve`` (``mhd.f90:303-325``)."""
        flux, expand = self.calc_flux()
        ff, ef = self.transform_flux_real_to_fourier(flux, expand)
        fnl = self.calc_rhs(ff, ef)
        self.rkt(irk, fnl)
        self.dealias()
        self.transform_uu_fourier_to_real()
        self.update_uu_prim_from_uu()

    def evolve(self):
        for irk in (1, 2, 3):
            self.stage(irk)

    def vardt_min(self):
        """Grid minimum of the CFL time step before the cfl factor (``mhd.f90:350-419``)."""
        p = self.p
        uu, pr = self.uu, self.uu_prim
        rho = uu[RHO]
        cs2 = p.adiabatic_index * pr[3] / rho
        sq = np.sqrt(rho)
        cax, cay, caz = uu[BX] / sq, uu[BY] / sq, uu[BZ] / sq
        ca2 = cax**2 + cay**2 + caz**2
        cms2 = cs2 + ca2
        s2 = math.sqrt(2.0)
        cmax = []
        for ca, u in ((cax, pr[0]), (cay, pr[1]), (caz, pr[2])):
            cns2 = np.sqrt(np.maximum(cms2**2 - 4 * cs2 * ca**2, 0.0))
            cf = np.sqrt(cms2 + cns2) / s2
            csl = np.sqrt(np.maximum(cms2 - cns2, 0.0)) / s2
            cmax.append(np.maximum.reduce([np.abs(u + cf), np.abs(u + csl), np.abs(u + ca),
                                           np.abs(u - cf), np.abs(u - csl), np.abs(u - ca), np.abs(u)]))
        if p.if_Hall:
            ch = p.ion_inertial_length / rho * np.maximum(np.maximum(uu[BX], uu[BY]), uu[BZ]) / min(
                self.dx, self.dy, self.dz)
            cmax = [np.maximum(c, ch) for c in cmax]
        with np.errstate(divide="ignore"):
            dtx = self.dx / cmax[0]
            dty = self.dy / cmax[1] * (self.radius / p.radius0)
            dtz = self.dz / cmax[2] * (self.radius / p.radius0)
        return float(np.min(np.minimum(np.minimum(dtx, dty), dtz)))

    def vardt(self):
        """dt = cfl * min, kept unless outside +-2 %, then rkt_init (``mhd.f90:422-428``)."""
        dtmin = self.vardt_min() * self.p.cfl
        if self.dt < 0.98 * dtmin or self.dt > 1.02 * dtmin:
            self.dt = dtmin
        self.rkt_init(self.dt)
        return self.dt

    def step(self):
        """One step as laps_step takes it: vardt; evolve; time += dt; evolve_radius(time) -
        the loop body of ``mhd.f90:245-285`` with its trailing vardt moved to the front (the
        first call plays the vardt before the loop, ``mhd.f90:135-136``)."""
        self.vardt()
        self.evolve()
        self.time = self.time + self.dt
        self.evolve_radius(self.time)

    def calc_max_divB(self):
        """max |ik . B_hat| over the spectral grid (``mhd.f90:522-570``)."""
        kx, ky, kz = self.ik()
        uf = self.uf
        d = 1j * kx * uf[BX] + 1j * ky * uf[BY] + 1j * kz * uf[BZ]
        return float(np.max(np.abs(d)))

    def calc_rms(self):
        """Means, variances and rho (u - <u>)^2 (``mhdrms.f90:53-126``); returns (ave, rms, rho_u2)."""
        uu, pr = self.uu, self.uu_prim
        n = uu[0].size
        f = [uu[RHO], pr[0], pr[1], pr[2], uu[BX], uu[BY], uu[BZ], pr[3]]
        ave = np.array([np.sum(a) for a in f]) / n
        sq = np.array([np.sum(a * a) for a in f]) / n
        rms = sq - ave**2
        rho_u2 = np.array([np.sum(uu[RHO] * (pr[i] - ave[1 + i]) ** 2) for i in range(3)]) / n
        return ave, rms, rho_u2

    def invariants(self):
        """Energy, cross-helicity and magnetic helicity (grid means).

        E_kin = <rho u^2>/2, E_mag = <B^2>/2, H_c = <u . B>, H_m = <A . B> with
        A_hat = i k x B_hat / k^2 (k != 0).  These histories are the solver's own additions
        (the reference prints only ``rms.dat``); the parity target for them is <=1e-9.
        """
        uu, pr = self.uu, self.uu_prim
        ekin = 0.5 * np.mean(uu[RHO] * (pr[0] ** 2 + pr[1] ** 2 + pr[2] ** 2))
        emag = 0.5 * np.mean(uu[BX] ** 2 + uu[BY] ** 2 + uu[BZ] ** 2)
        hc = np.mean(pr[0] * uu[BX] + pr[1] * uu[BY] + pr[2] * uu[BZ])
        hm = magnetic_helicity(self.uf[BX:BZ + 1], *self.ik(), self.p.nx)
        return np.array([ekin, emag, hc, hm])


def magnetic_helicity(bf, kx, ky, kz, nx):
    """<A . B> from the half spectrum with the Coulomb-gauge A_hat = i k x B_hat / k^2.

    Parseval on a half spectrum: modes 0 < kx < nx/2 count twice (their conjugates are
    not stored), kx = 0 and kx = nx/2 once.
    """
    k2 = kx * kx + ky * ky + kz * kz
    with np.errstate(divide="ignore", invalid="ignore"):
        inv = np.where(k2 > 0, 1.0 / np.where(k2 > 0, k2, 1.0), 0.0)
    ax = 1j * (ky * bf[2] - kz * bf[1]) * inv
    ay = 1j * (kz * bf[0] - kx * bf[2]) * inv
    az = 1j * (kx * bf[1] - ky * bf[0]) * inv
    dens = (ax * np.conj(bf[0]) + ay * np.conj(bf[1]) + az * np.conj(bf[2])).real
    w = np.full(dens.shape[-1], 2.0)
    w[0] = 1.0
    if nx % 2 == 0:
        w[-1] = 1.0
    return float(np.sum(dens * w[None, None, :]))


def shell_spectra(uu: np.ndarray, Lx: float, Ly: float, Lz: float, nshell: int):
    """Shell energy spectra E_u(k) = 1/2 sum |u_hat|^2 and E_b(k) = 1/2 sum |B_hat|^2.

    u = (rho u)/rho from the conserved real fields ``uu[0:4]``, B = ``uu[4:7]``; hats are the
    reference's forward transform (divided by n per axis, ``fftw.f90:42-71``), so the shells
    sum to <u^2>/2 and <B^2>/2.  Shell s holds the modes with round(|k|/dk) = s, |k| from the
    grid's unscaled wave numbers (``mhdinit.f90:88-115``) and dk = 2 pi / max(L) over the
    axes with more than one point; modes beyond the last shell are dropped.  The reference
    post-processes |B_hat|^2 the same way with numpy's fftn
    (``data_process/3D_Python/fourier_analysis.py:150-200``); the shell binning is this
    solver's own.  A half spectrum counts modes 0 < kx < nx/2 twice.
    """
    nz, ny, nx = uu.shape[-3:]
    u = uu[1:4] / uu[0]
    uh = forward_3d(u)
    bh = forward_3d(uu[4:7])
    kx = wave_numbers(nx, Lx)[: nx // 2 + 1]
    ky = wave_numbers(ny, Ly)
    kz = wave_numbers(nz, Lz) if nz > 1 else np.zeros(1)
    Ls = [L for L, n in ((Lx, nx), (Ly, ny), (Lz, nz)) if n > 1]
    dk = 2 * PI / max(Ls)
    kk = np.sqrt(kz[:, None, None] ** 2 + ky[None, :, None] ** 2 + kx[None, None, :] ** 2)
    shell = np.floor(kk / dk + 0.5).astype(np.int64)
    w = np.where((np.arange(nx // 2 + 1) == 0) | (2 * np.arange(nx // 2 + 1) == nx), 1.0, 2.0)[None, None, :]
    eu = 0.5 * w * np.sum(np.abs(uh) ** 2, axis=0)
    eb = 0.5 * w * np.sum(np.abs(bh) ** 2, axis=0)
    keep = shell < nshell
    return (np.bincount(shell[keep], eu[keep], minlength=nshell)[:nshell],
            np.bincount(shell[keep], eb[keep], minlength=nshell)[:nshell])


def params_from(n, kw) -> Params3D:
    """Params3D for an n^3 (or (nx, ny, nz)) grid from C-ABI-style keyword values."""
    nx, ny, nz = (n, n, n) if np.isscalar(n) else n
    p = Params3D(nx=nx, ny=ny, nz=nz)
    for k, v in kw.items():
        if not hasattr(p, k):
            continue
        cur = getattr(p, k)
        setattr(p, k, bool(v) if isinstance(cur, bool) else type(cur)(v))
    return p


def restart(n, kw, prim, t0=0.0) -> Laps3DC:
    """Start as the reference's restart path does: read primitives, evolve_radius(t0),
    conserve, forward transform (src_compressible/mhd.f90:101-122)."""
    o = Laps3DC(params_from(n, kw))
    o.initial_calc_conserve_variable(prim)
    o.time = t0
    o.evolve_radius(t0)
    o.transform_uu_real_to_fourier()
    return o


# ============================================================================ 2-D compressible
@dataclasses.dataclass
class Params2D(Params3D):
    """Namelist values of the 2-D compressible code (``src_compressible/2D/mhd.f90:33-43``);
    nz = 1.  ``if_limit_dt_increase`` and the vardt cadence ``dstep_calcdt``
    (``src_compressible/2D/mhd.f90:20,23``) are 2-D only."""

    nz: int = 1
    if_z_radial: bool = False
    if_limit_dt_increase: bool = False
    dstep_calcdt: int = 20


class Laps2DC(Laps3DC):
    """2-D compressible solver: the 3-D routines with kz = 0 and the 2-D differences
    (``src_compressible/2D/``): radial-z expansion geometry, square dealias option 3, the
    explicit-eta CFL term and vardt every ``dstep_calcdt`` steps."""

    def __init__(self, p: Params2D):
        assert p.nz == 1
        super().__init__(p)
        self.wz = np.zeros(1)
        self.zrad = bool(p.if_AEB and p.if_z_radial)
        self.k_square = self.wx[None, None, :] ** 2 + self.wy[None, :, None] ** 2
        self.dz = None
        self.istep = 0

    def _init_dealias(self):
        p = self.p
        if p.dealias_option == 1:
            rx = (self.wx * p.Lx / (2 * PI * p.nx)) ** 2
            ry = (self.wy * p.Ly / (2 * PI * p.ny)) ** 2
            rad = np.sqrt(rx[None, None, :] + ry[None, :, None])
            self.keep = ~(rad > 1.0 / 3.0)
        elif p.dealias_option == 3:  # square 2/3 truncation, 2D/dealiasing.f90:102-117
            rx = np.abs(self.wx * p.Lx / (2 * PI * p.nx))
            ry = np.abs(self.wy * p.Ly / (2 * PI * p.ny))
            self.keep = ~((rx[None, None, :] > 1.0 / 3.0) | (ry[None, :, None] > 1.0 / 3.0))
        elif p.dealias_option == 2:
            super()._init_dealias()
            self.filtz = np.ones(1)

    def dealias(self):
        p = self.p
        if p.dealias_option in (1, 3):
            self.uf[:, ~self.keep] = 0.0
        elif p.dealias_option == 2:
            self.uf = (self.uf * self.filtx[None, None, None, :]) * self.filty[None, None, :, None]

    def evolve_radius(self, t):
        """``src_compressible/2D/AEBmod.f90``: k^2 without kz; radial-z scales kx too."""
        p = self.p
        self.radius = p.radius0 + self.Ur0 * t
        self.tau_exp = self._tau(self.radius)
        kx = self.wx[None, None, :]
        ky = self.wy[None, :, None]
        R0, R = p.radius0, self.radius
        if p.if_corotating:
            c, s = self.cos_cor, self.sin_cor
            self.k_square = (kx**2 * (c**2 + (s * R0 / R) ** 2) + ky**2 * (s**2 + (c * R0 / R) ** 2)
                             + kx * ky * 2 * c * s * (1 - (R0 / R) ** 2))
        elif p.if_z_radial:
            self.k_square = (kx * R0 / R) ** 2 + (ky * R0 / R) ** 2
        else:
            self.k_square = kx**2 + (ky * R0 / R) ** 2

    def ik(self):
        """``src_compressible/2D/mhdrhs.f90:272-288``: kz = 0; radial-z scales kx by R0/R."""
        kx, ky, kz = super().ik()
        if self.zrad and not (self.p.if_AEB and self.p.if_corotating):
            kx = kx * self.p.radius0 / self.radius
        return kx, ky, np.zeros_like(kz)

    def expansion_coefficients(self):
        """(rho, rho u, B) damping factors of calc_rhs (``2D/mhdrhs.f90:319-343``)."""
        if self.zrad:
            return (2.0, 3.0, 3.0, 2.0, 1.0, 1.0, 2.0)
        return (2.0, 2.0, 3.0, 3.0, 2.0, 1.0, 1.0)

    def expand_term(self, P, Bx, By, Bz, uu, ux, uy, uz, g, tau):
        if self.zrad:  # 2D/mhdrhs.f90:96-100
            return (-2 * g / (g - 1) * P / tau - (Bx**2 + By**2 + 2.0 * Bz**2) / tau
                    - (2 * uu[MX] * ux + 2 * uu[MY] * uy + uu[MZ] * uz) / tau)
        return super().expand_term(P, Bx, By, Bz, uu, ux, uy, uz, g, tau)

    def vardt_min(self):
        """``src_compressible/2D/mhd.f90:294-394``: x and y only, explicit-eta term, radial x."""
        p = self.p
        uu, pr = self.uu, self.uu_prim
        rho = uu[RHO]
        cs2 = p.adiabatic_index * pr[3] / rho
        sq = np.sqrt(rho)
        cax, cay, caz = uu[BX] / sq, uu[BY] / sq, uu[BZ] / sq
        ca2 = cax**2 + cay**2 + caz**2
        cms2 = cs2 + ca2
        s2 = math.sqrt(2.0)
        cmax = []
        for ca, u in ((cax, pr[0]), (cay, pr[1])):
            cns2 = np.sqrt(np.maximum(cms2**2 - 4 * cs2 * ca**2, 0.0))
            cf = np.sqrt(cms2 + cns2) / s2
            csl = np.sqrt(np.maximum(cms2 - cns2, 0.0)) / s2
            cmax.append(np.maximum.reduce([np.abs(u + cf), np.abs(u + csl), np.abs(u + ca),
                                           np.abs(u - cf), np.abs(u - csl), np.abs(u - ca), np.abs(u)]))
        if p.if_resis and p.if_resis_exp:
            cmax = [np.maximum(cmax[0], p.resistivity / self.dx), np.maximum(cmax[1], p.resistivity / self.dy)]
        if p.if_Hall:
            ch = p.ion_inertial_length / rho * np.maximum(np.maximum(uu[BX], uu[BY]), uu[BZ]) / min(self.dx, self.dy)
            cmax = [np.maximum(c, ch) for c in cmax]
        with np.errstate(divide="ignore"):
            dtx = self.dx / cmax[0]
            if p.if_AEB and p.if_z_radial:
                dtx = dtx * (self.radius / p.radius0)
            dty = self.dy / cmax[1] * (self.radius / p.radius0)
        return float(np.min(np.minimum(dtx, dty)))

    def vardt(self):
        """dt = cfl * min; +-2 % hysteresis, or with if_limit_dt_increase only a decrease (or
        the first call) replaces dt (``2D/mhd.f90:396-405``)."""
        dtmin = self.vardt_min() * self.p.cfl
        if self.p.if_limit_dt_increase:
            if self.dt == 0.0 or self.dt > 1.02 * dtmin:
                self.dt = dtmin
        elif self.dt < 0.98 * dtmin or self.dt > 1.02 * dtmin:
            self.dt = dtmin
        self.rkt_init(self.dt)
        return self.dt

    def step(self):
        """Loop body of ``2D/mhd.f90:196-240``, with vardt at the front of the step when
        istep is a multiple of dstep_calcdt (istep = 0 is the call before the loop)."""
        if self.istep % self.p.dstep_calcdt == 0:
            self.vardt()
        self.evolve()
        self.time = self.time + self.dt
        self.istep += 1
        self.evolve_radius(self.time)


def restart2d(n, kw, prim, t0=0.0) -> Laps2DC:
    nx, ny = (n, n) if np.isscalar(n) else n[:2]
    p = Params2D(nx=nx, ny=ny, nz=1)
    for k, v in kw.items():
        if hasattr(p, k):
            cur = getattr(p, k)
            setattr(p, k, bool(v) if isinstance(cur, bool) else type(cur)(v))
    o = Laps2DC(p)
    o.initial_calc_conserve_variable(prim)
    o.time = t0
    o.evolve_radius(t0)
    o.transform_uu_real_to_fourier()
    return o


# ============================================================================ 3-D incompressible
@dataclasses.dataclass
class Params3DI(Params3D):
    """``src_incompressible``: rho0 is the module default of mhdinit.f90:15 (not a namelist
    value); it divides the velocity gradient and decays with the expanding box."""

    rho0: float = 1.0


class Laps3DI(Laps3DC):
    """3-D incompressible solver (``src_incompressible/``).  State slots: 1 rho, 2:4 rho u,
    5:7 B, 8 pressure p (no energy); uu_prim = u."""

    def initial_calc_conserve_variable(self, prim):
        """rho u = rho * u; p kept (``src_incompressible/mhdinit.f90:1031-1042``)."""
        uu = np.array(prim, dtype=np.float64, copy=True)
        self.uu_prim = uu[1:4].copy()
        uu[1] = uu[0] * self.uu_prim[0]
        uu[2] = uu[0] * self.uu_prim[1]
        uu[3] = uu[0] * self.uu_prim[2]
        self.uu = uu
        self.rho0 = self.p.rho0

    def update_uu_prim_from_uu(self):
        """``src_incompressible/mhdrhs.f90:235-242``."""
        uu = self.uu
        self.uu_prim = np.stack([uu[1] / uu[0], uu[2] / uu[0], uu[3] / uu[0]])

    def calc_gradient_velocity_real(self):
        """grad(rho u)/rho0, 9 inverse transforms (``src_incompressible/mhdrhs.f90:312-391``):
        order d(ux)/dx, d(ux)/dy, d(ux)/dz, d(uy)/dx, ..."""
        kx, ky, kz = self.ik()
        uf = self.uf
        gf = []
        for v in (MX, MY, MZ):
            for k in (kx, ky, kz):
                gf.append(1j * k * uf[v])
        gf = np.stack(gf) / self.rho0
        return inverse_3d(gf, self.p.nx)

    def stage(self, irk):
        """One RK stage of the incompressible evolve (``src_incompressible/mhd.f90:323-363``)."""
        p = self.p
        self.transform_uu_real_to_fourier()
        J = self.calc_current_density_real()
        G = self.calc_gradient_velocity_real()
        uu = self.uu
        # calc_flux_for_pressure, src_incompressible/mhdrhs.f90:393-437
        fp = np.stack([
            -uu[MX] * G[0] - uu[MY] * G[1] - uu[MZ] * G[2] + J[1] * uu[BZ] - J[2] * uu[BY],
            -uu[MX] * G[3] - uu[MY] * G[4] - uu[MZ] * G[5] + J[2] * uu[BX] - J[0] * uu[BZ],
            -uu[MX] * G[6] - uu[MY] * G[7] - uu[MZ] * G[8] + J[0] * uu[BY] - J[1] * uu[BX],
        ])
        fpf = forward_3d(fp)
        kx, ky, kz = self.ik()
        k2 = self.k_square
        small = k2 < 1e-10
        with np.errstate(divide="ignore", invalid="ignore"):
            kdot = (1j * kx * fpf[0] + 1j * ky * fpf[1] + 1j * kz * fpf[2]) / np.where(small, 1.0, k2)
        kdot = np.where(small, 0.0, kdot)
        # calc_pressure_fourier, :468-518
        self.uf[EN] = np.where(small, 0.0, -kdot)
        # calc_flux (electric field), :25-84
        pr = self.uu_prim
        E = np.stack([pr[2] * uu[BY] - pr[1] * uu[BZ], pr[0] * uu[BZ] - pr[2] * uu[BX], pr[1] * uu[BX] - pr[0] * uu[BY]])
        if p.if_Hall:
            di = p.ion_inertial_length
            E[0] = E[0] + di / uu[RHO] * (J[1] * uu[BZ] - J[2] * uu[BY])
            E[1] = E[1] + di / uu[RHO] * (J[2] * uu[BX] - J[0] * uu[BZ])
            E[2] = E[2] + di / uu[RHO] * (J[0] * uu[BY] - J[1] * uu[BX])
        Ef = forward_3d(E)
        # calc_rhs, :117-232
        uf = self.uf
        fnl = np.zeros_like(uf)
        fnl[1] = np.where(small, 0.0, fpf[0] + kdot * 1j * kx)
        fnl[2] = np.where(small, 0.0, fpf[1] + kdot * 1j * ky)
        fnl[3] = np.where(small, 0.0, fpf[2] + kdot * 1j * kz)
        fnl[4] = 1j * kz * Ef[1] - 1j * ky * Ef[2]
        fnl[5] = 1j * kx * Ef[2] - 1j * kz * Ef[0]
        fnl[6] = 1j * ky * Ef[0] - 1j * kx * Ef[1]
        if p.if_AEB:
            tau = self.tau_exp
            for v, c in ((0, 2.0), (1, 2.0), (2, 3.0), (3, 3.0), (4, 2.0), (5, 1.0), (6, 1.0)):
                fnl[v] = fnl[v] - c * uf[v] / tau
            fnl[7] = fnl[7] - 2.0 * p.adiabatic_index * uf[7] / tau
        if p.if_visc and p.if_visc_exp:
            for v in (1, 2, 3):
                fnl[v] = fnl[v] - p.viscosity * uf[v] * k2
        if p.if_resis and p.if_resis_exp:
            m = np.ones(k2.shape, bool)
            if p.if_conserve_background:
                m[0, :, 0] = False
            for v in (4, 5, 6):
                fnl[v] = np.where(m, fnl[v] - p.resistivity * uf[v] * k2, fnl[v])
        self.rkt(irk, fnl)
        self.dealias()
        self.transform_uu_fourier_to_real()
        self.update_uu_prim_from_uu()

    def evolve(self):
        for irk in (1, 2, 3):
            self.stage(irk)
        # update_rho_p (src_incompressible/AEBmod.f90:123-134), at the step's start radius
        self.rho0 = self.rho0 * (self.p.radius0 / self.radius) ** 2

    def vardt_min(self):
        """Alfven-only CFL (``src_incompressible/mhd.f90:394-463``)."""
        p = self.p
        uu, pr = self.uu, self.uu_prim
        rho = uu[RHO]
        sq = np.sqrt(rho)
        cmax = []
        for b, u in ((BX, pr[0]), (BY, pr[1]), (BZ, pr[2])):
            ca = uu[b] / sq
            cmax.append(np.maximum.reduce([np.abs(u + ca), np.abs(u - ca), np.abs(u)]))
        if p.if_Hall:
            ch = p.ion_inertial_length / rho * np.maximum(np.maximum(uu[BX], uu[BY]), uu[BZ]) / min(
                self.dx, self.dy, self.dz)
            cmax = [np.maximum(c, ch) for c in cmax]
        with np.errstate(divide="ignore"):
            dtx = self.dx / cmax[0]
            dty = self.dy / cmax[1] * (self.radius / p.radius0)
            dtz = self.dz / cmax[2] * (self.radius / p.radius0)
        return float(np.min(np.minimum(np.minimum(dtx, dty), dtz)))

    def calc_rms(self):
        """``src_incompressible/mhdrms.f90:47-120``.  Its p columns read uu_prim(:,:,:,4),
        beyond the 3 components uu_prim has here, and are undefined; the pressure held in
        slot 8 is reported there instead."""
        uu, pr = self.uu, self.uu_prim
        n = uu[0].size
        f = [uu[RHO], pr[0], pr[1], pr[2], uu[BX], uu[BY], uu[BZ], uu[EN]]
        ave = np.array([np.sum(a) for a in f]) / n
        sq = np.array([np.sum(a * a) for a in f]) / n
        rms = sq - ave**2
        rho_u2 = np.array([np.sum(uu[RHO] * (pr[i] - ave[1 + i]) ** 2) for i in range(3)]) / n
        return ave, rms, rho_u2

    def div_maxima(self):
        """max |div B| and max |div(rho u)|/rho0 in real space (calc_divB_real,
        calc_divV_real and their maxima: src_incompressible/mhdrhs.f90:532-648,
        mhd.f90:672-732)."""
        kx, ky, kz = self.ik()
        uf = self.uf
        db = inverse_3d(1j * kx * uf[BX] + 1j * ky * uf[BY] + 1j * kz * uf[BZ], self.p.nx)
        dv = inverse_3d((1j * kx * uf[MX] + 1j * ky * uf[MY] + 1j * kz * uf[MZ]) / self.rho0, self.p.nx)
        return float(np.max(np.abs(db))), float(np.max(np.abs(dv)))

    def invariants(self):
        uu, pr = self.uu, self.uu_prim
        ekin = 0.5 * np.mean(uu[RHO] * (pr[0] ** 2 + pr[1] ** 2 + pr[2] ** 2))
        emag = 0.5 * np.mean(uu[BX] ** 2 + uu[BY] ** 2 + uu[BZ] ** 2)
        hc = np.mean(pr[0] * uu[BX] + pr[1] * uu[BY] + pr[2] * uu[BZ])
        hm = magnetic_helicity(self.uf[BX:BZ + 1], *self.ik(), self.p.nx)
        return np.array([ekin, emag, hc, hm])


def restart3di(n, kw, prim, t0=0.0) -> Laps3DI:
    nx, ny, nz = (n, n, n) if np.isscalar(n) else n
    p = Params3DI(nx=nx, ny=ny, nz=nz)
    for k, v in kw.items():
        if hasattr(p, k):
            cur = getattr(p, k)
            setattr(p, k, bool(v) if isinstance(cur, bool) else type(cur)(v))
    o = Laps3DI(p)
    o.initial_calc_conserve_variable(prim)
    o.time = t0
    o.evolve_radius(t0)
    o.transform_uu_real_to_fourier()
    return o
