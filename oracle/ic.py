"""CPU restatement of the reference's fresh-start initial conditions (test infrastructure).

This module is the oracle of ``laps_init_fields``: the parity tests compare the device's
generated state with the arrays built here.  Nothing in the product imports it.

It follows, point by point and mode by mode in float64 numpy:
  - ``background_fields_initialize``  src_compressible/mhdinit.f90:183-299
    (src_incompressible/mhdinit.f90:190-300: the same cases 0-4, no case 5);
  - ``perturbation_initialize``       src_compressible/mhdinit.f90:302-1036 for ipert 1
    (:328-342; the incompressible form src_incompressible/mhdinit.f90:318-333), 6 (:487-688),
    7 (:690-930) and 8 (:931-1019), the random-phase sums evaluated directly as sums of
    cosines over the grid, as the reference does.
The reference draws the phases of ipert 6 and 7 with the compiler's ``random_number``
(mhdinit.f90:495-498,566-569,703-727); here they are an argument, in the layout of the
reference's ``phs`` arrays (index expressions at :523-526, :594-597, :762-769, 0-based).
Arrays are primitive ``(rho, ux, uy, uz, Bx, By, Bz, p)`` stored ``[ivar, iz, iy, ix]``.
"""
from __future__ import annotations

import math

import numpy as np

PI = 3.141592653589793  # the reference's module constant (mhdinit.f90:7)


def ic_default() -> dict:
    """The reference's module initialisers (mhdinit.f90:13-14,48-55)."""
    return dict(ifield=0, ipert=0, T0=1.0, rho0=1.0, B0=1.0, a0=0.05, U_fast=0.0, U_slow=0.0, n_fast=0.0,
                n_slow=0.0, press0=0.0, shear_width=0.0, bx0=0.0, by0=0.0, bz0=0.0, db0=0.0, in_out_ratio=1.0,
                dv0=0.0, drho0=0.0, nmodex=16, nmodey=16, nmodez=16, wave_number_jet=1, jet_width=1.0, Vjet=0.3,
                B0_SB=0.0, dB_SB=0.0, R0_SB=0.0, R1_SB=0.0, H_SB=0.0, Rm_SB=0.0, Rd_SB=0.0)


def nphases(ic: dict) -> int:
    """Phases ipert 6 and 7 read (outward + inward waves; u, B, rho)."""
    mx, my, mz = ic["nmodex"], ic["nmodey"], ic["nmodez"]
    if ic["ipert"] == 6:
        return 2 * mx * (2 * my + 1) * (2 * mz + 1)
    if ic["ipert"] == 7:
        return 3 * (2 * mx + 1) * (2 * my + 1) * (2 * mz + 1)
    return 0


def grids(shape, L):
    nz, ny, nx = shape
    Lx, Ly, Lz = L
    # xgrid(ix) = (ix - 1) * dx, mhdinit.f90:84-104
    return (np.arange(nx) * (Lx / nx), np.arange(ny) * (Ly / ny), np.arange(nz) * (Lz / nz))


def background(shape, L, ic: dict, incompressible=False) -> np.ndarray:
    """background_fields_initialize, mhdinit.f90:183-299."""
    nz, ny, nx = shape
    Lx, Ly, Lz = L
    x, y, z = grids(shape, L)
    u = np.zeros((8, nz, ny, nx))
    T0, rho0, B0, a0 = ic["T0"], ic["rho0"], ic["B0"], ic["a0"]
    ninf = 1.0
    u[0] = rho0
    u[7] = rho0 * T0
    f = ic["ifield"]
    if f == 1:  # :205-222, double current sheet Bx(z), density balances the pressure
        zlow, zup, zc = 0.25 * Lz, 0.75 * Lz, 0.5 * Lz
        zz = np.where(z < zc, z - zlow, z - zup)
        sg = np.where(z < zc, 1.0, -1.0)
        u[4] = (sg * B0 * np.tanh(zz / a0))[:, None, None]
        u[0] = (ninf + B0**2 / 2.0 / T0 / np.cosh(zz / a0) ** 2)[:, None, None]
        u[7] = u[0] * T0
    elif f == 2:  # :224-248, double Harris shear ux(y), rho(y)
        ylow, yup, yc = 0.25 * Ly, 0.75 * Ly, 0.5 * Ly
        a = Ly * 0.5 * ic["shear_width"]
        yy = np.where(y < yc, y - ylow, y - yup)
        sg = np.where(y < yc, 1.0, -1.0)
        t = np.tanh(yy / a)
        Uf, Us, nf, ns = ic["U_fast"], ic["U_slow"], ic["n_fast"], ic["n_slow"]
        u[1] = (sg * 0.5 * (Uf - Us) * t + 0.5 * (Uf + Us))[None, :, None]
        u[0] = (sg * 0.5 * (nf - ns) * t + 0.5 * (nf + ns))[None, :, None]
        u[7] = ic["press0"]
        u[4] = ic["bx0"]
        u[5] = ic["by0"]
    elif f == 3:  # :250-255, uniform B
        u[4], u[5], u[6], u[7] = ic["bx0"], ic["by0"], ic["bz0"], ic["press0"]
    elif f == 4:  # :258-273, double current sheet Bx(y), pressure balance by temperature
        ylow, yup, yc = 0.25 * Ly, 0.75 * Ly, 0.5 * Ly
        yy = np.where(y < yc, y - ylow, y - yup)
        sg = np.where(y < yc, 1.0, -1.0)
        bx = sg * B0 * np.tanh(yy / a0)
        u[4] = bx[None, :, None]
        u[7] = (ic["press0"] - 0.5 * bx**2)[None, :, None]
        u[0] = ninf
    elif f == 5 and not incompressible:  # :275-292, jet along x
        u[4], u[5], u[6], u[7] = ic["bx0"], ic["by0"], ic["bz0"], ic["press0"]
        r = np.sqrt((z[:, None] - Lz / 2) ** 2 + (y[None, :] - Ly / 2) ** 2)
        u[1] = (ic["Vjet"] / 2 * (1 - np.tanh((r - 1) / 0.1)))[:, :, None]
    return u


def _sign(v):
    return math.copysign(1.0, v)  # Fortran sign(1.0, v)


def perturb(u: np.ndarray, L, ic: dict, phases=None, incompressible=False, cor_angle=0.0) -> np.ndarray:
    """perturbation_initialize for ipert 1, 6, 7, 8 (mhdinit.f90:302-1036), added to u."""
    nz, ny, nx = u.shape[1:]
    Lx, Ly, Lz = L
    x, y, z = grids(u.shape[1:], L)
    ip = ic["ipert"]
    sa, ca = math.sin(cor_angle), math.cos(cor_angle)
    db0 = ic["db0"]
    if ip == 1:
        if incompressible:  # src_incompressible/mhdinit.f90:318-333
            kx = 2 * PI / Lx
            s, c = np.sin(kx * x), np.cos(kx * x)
            sr = np.sqrt(u[0])
            u[6] = u[6] - db0 * sr * s
            u[3] = u[3] + db0 * s
            u[1] = u[1] + db0 * c * sa
            u[4] = u[4] - db0 * sr * c * sa
            u[2] = u[2] + db0 * c * ca
            u[5] = u[5] - db0 * sr * c * ca
        else:  # src_compressible/mhdinit.f90:328-342
            kx = 2 * PI / Lx * ic["wave_number_jet"]
            s, c = np.sin(kx * x), np.cos(kx * x)
            sr = np.sqrt(u[0])
            u[6] = u[6] - db0 * s
            u[3] = u[3] + db0 / sr * s
            u[1] = u[1] + db0 / sr * c * sa
            u[4] = u[4] - db0 * c * sa
            u[2] = u[2] + db0 / sr * c * ca
            u[5] = u[5] - db0 * c * ca
    elif ip == 6:
        mx, my, mz = ic["nmodex"], ic["nmodey"], ic["nmodez"]
        nm = mx * (2 * my + 1) * (2 * mz + 1)
        ph = np.asarray(phases, dtype=np.float64)
        sgn = _sign(ic["bx0"])
        Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
        for wave, (dirx, su, amp_io, off) in enumerate(((1, -1.0, 1.0, 0), (-1, 1.0, ic["in_out_ratio"], nm))):
            # outward (:500-560) then inward (:571-633) waves
            for ikx in range(1, mx + 1):
                kx = dirx * ikx * 2 * PI / Lx
                ax = math.sqrt(1 / float(abs(ikx)))
                for iky in range(-my, my + 1):
                    ky = iky * 2 * PI / Ly
                    ay = 1.0 if iky == 0 else math.sqrt(1 / float(abs(iky)))
                    for ikz in range(-mz, mz + 1):
                        kz = ikz * 2 * PI / Lz
                        az = 1.0 if ikz == 0 else math.sqrt(1 / float(abs(ikz)))
                        p0 = ph[off + ((ikx - 1) * (2 * my + 1) + iky + my) * (2 * mz + 1) + ikz + mz]
                        pph = kx * X + ky * Y + kz * Z + p0
                        a = ax * ay * az * amp_io
                        if iky == 0 and ikz == 0:
                            cp, sp = np.cos(pph), np.sin(pph)
                            u[5] += db0 * cp * a
                            u[6] += db0 * sp * a
                            u[2] += su * sgn * db0 * cp * a
                            u[3] += su * sgn * db0 * sp * a
                        else:
                            dby = db0 * kz / math.sqrt(ky**2 + kz**2)
                            dbz = -db0 * ky / math.sqrt(ky**2 + kz**2)
                            cp = np.cos(pph)
                            u[5] += dby * cp * a
                            u[6] += dbz * cp * a
                            u[2] += su * sgn * dby * cp * a
                            u[3] += su * sgn * dbz * cp * a
    elif ip == 7:
        mx, my, mz = ic["nmodex"], ic["nmodey"], ic["nmodez"]
        nm = (2 * mx + 1) * (2 * my + 1) * (2 * mz + 1)
        ph = np.asarray(phases, dtype=np.float64)
        corr = -0.05
        bx0, by0, bz0 = ic["bx0"], ic["by0"], ic["bz0"]
        dv0, drho0 = ic["dv0"], ic["drho0"]
        Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
        for ikx in range(0, mx + 1):
            kx = ikx * 2 * PI / Lx
            for iky in range(-my, my + 1):
                ky = iky * 2 * PI / Ly
                for ikz in range(-mz, mz + 1):
                    kz = ikz * 2 * PI / Lz
                    if (ikx == 0 and iky < 0) or (ikx == 0 and iky == 0 and ikz <= 0):
                        continue
                    kr = math.sqrt(float(ikx**2 + iky**2 + ikz**2))
                    if kr > max(mx, my, mz):
                        continue
                    kmod = math.sqrt(kx**2 + ky**2 + kz**2)
                    B0mod = math.sqrt(bx0**2 + by0**2 + bz0**2)
                    d = ((ky * bz0 - kz * by0) / kmod / B0mod, (kz * bx0 - kx * bz0) / kmod / B0mod,
                         (kx * by0 - ky * bx0) / kmod / B0mod)
                    j = ((ikx + mx) * (2 * my + 1) + iky + my) * (2 * mz + 1) + ikz + mz
                    ph0, ph1, ph2 = ph[j], ph[nm + j], ph[2 * nm + j]
                    kr3 = math.sqrt(kr**3)
                    base = kx * X + ky * Y + kz * Z
                    c0, c1, c2 = np.cos(base + ph0), np.cos(base + ph1), np.cos(base + ph2)
                    for c in range(3):
                        u[1 + c] += math.sqrt(1 - corr**2) * dv0 * c0 / kr3 * d[c]
                    for c in range(3):
                        u[4 + c] += db0 * c1 / kr3 * d[c]
                    for c in range(3):
                        u[1 + c] += corr * dv0 * c1 / kr3 * d[c]
                    u[0] += drho0 * c2 / kr3
    elif ip == 8:
        _switchback(u, L, ic)
    return u


def _switchback(u, L, ic):
    """ipert 8, mhdinit.f90:931-1019 (a magnetic switchback along x with anti-correlated u)."""
    from math import erf

    Lx, Ly, Lz = L
    x, y, z = grids(u.shape[1:], L)
    B0s, dBs, R0s, R1s, Hs, Rms, Rds = (ic[k] for k in ("B0_SB", "dB_SB", "R0_SB", "R1_SB", "H_SB", "Rm_SB", "Rd_SB"))
    verf = np.vectorize(erf)
    Cs = -(math.exp(-((R0s / R1s) ** 2)) + math.sqrt(PI) * R0s / R1s * erf(R0s / R1s))
    Z, Y, X = np.meshgrid(z - Lz / 2, y - Ly / 2, x - Lx / 2, indexing="ij")
    r = np.sqrt(Y**2 + Z**2)
    Bz0 = B0s + dBs * np.exp(-(((r - R0s) / R1s) ** 2))
    Bz = B0s + dBs * np.exp(-(((r - R0s) / R1s) ** 2) - (X / Hs) ** 2)
    core = r < 1e-8
    rs = np.where(core, 1.0, r)
    phi = np.where(core, 0.0, np.arctan2(Z, Y))
    G = np.exp(-(((rs - R0s) / R1s) ** 2)) + math.sqrt(PI) * R0s / R1s * verf((R0s - rs) / R1s) + Cs
    Br = -dBs * (X * R1s**2) / (rs * Hs**2) * np.exp(-((X / Hs) ** 2)) * G
    inner = rs < Rms
    p = np.where(inner, 1.0, np.exp(-(((rs - Rms) / Rds) ** 2)))
    dpdr = np.where(inner, 0.0, -2 * (rs - Rms) / Rds**2 * p)
    q = np.where(inner, 1.0,
                 Bz0 / Bz * (1 + 1 / Bz0 * (p * (Bz - Bz0) - (dpdr * dBs * R1s**2 / rs * G * 0.5 * (np.exp(-((X / Hs) ** 2)) - 1)))))
    Br = Br * p
    Bzq = Bz * q
    under = Bzq**2 + Br**2 < B0s**2
    Bphi = np.where(under, np.sqrt(np.where(under, B0s**2 - Br**2 - Bzq**2, 0.0)), 0.0)
    dp = np.where(under, 0.0, -0.5 * (Bzq**2 + Br**2 - B0s**2))
    # the core line r < 1e-8 keeps Bz unscaled, Br = Bphi = 0 and the pressure unchanged
    Br = np.where(core, 0.0, Br)
    Bphi = np.where(core, 0.0, Bphi)
    Bzf = np.where(core, Bz, Bzq)
    dp = np.where(core, 0.0, dp)
    u[7] += dp
    Bx = Br * np.cos(phi) - Bphi * np.sin(phi)
    By = Br * np.sin(phi) + Bphi * np.cos(phi)
    u[4] += Bzf
    u[5] += Bx
    u[6] += By
    sr = np.sqrt(u[0])
    u[1] -= u[4] / sr
    u[2] -= u[5] / sr
    u[3] -= u[6] / sr


def initial_fields(shape, L, ic: dict, phases=None, incompressible=False, cor_angle=0.0) -> np.ndarray:
    """background + perturbation (mhd.f90:110-117): primitive fields [8, nz, ny, nx]."""
    u = background(shape, L, ic, incompressible)
    return perturb(u, L, ic, phases, incompressible, cor_angle)
