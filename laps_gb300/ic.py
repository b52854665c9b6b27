"""Seeded initial conditions in the reference's primitive layout.

The arrays returned here are what LAPS reads back from ``outNNN.dat`` through its restart
path (``src_compressible/restart.f90:17-63``): primitive variables
``(rho, ux, uy, uz, Bx, By, Bz, p)`` in Fortran order ``(nx, ny, nz, 8)``, stored in numpy
as ``[ivar, iz, iy, ix]``.  The conserved form is formed afterwards by
``initial_calc_conserve_variable`` (``src_compressible/mhdinit.f90:1038-1056``), on the GPU
by ``laps_upload_state``.
"""
from __future__ import annotations

import math

import numpy as np

PI = 3.141592653589793


def random_phase_spectrum(shape, L, kmin, kmax, alpha, rng):
    """One divergence-free random vector field with |k|^alpha amplitudes on kmin <= |k| <= kmax.

    Integer wave vectors (in units of 2 pi / L) inside the shell get an independent complex
    Gaussian direction with a uniform random phase and amplitude |k|^alpha, are projected
    onto the plane perpendicular to k, and are transformed to real space (the half
    spectrum's implied Hermitian partner makes the field real).  Returns ``[3, nz, ny, nx]``
    with zero mean and unit rms of |v|.
    """
    nz, ny, nx = shape
    Lx, Ly, Lz = L
    mx = np.arange(nx // 2 + 1)
    my = np.fft.fftfreq(ny, 1.0 / ny)
    mz = np.fft.fftfreq(nz, 1.0 / nz)
    KZ, KY, KX = np.meshgrid(mz * (2 * PI / Lz), my * (2 * PI / Ly), mx * (2 * PI / Lx), indexing="ij")
    MZ, MY, MX = np.meshgrid(mz, my, mx, indexing="ij")
    kmag = np.sqrt(MX**2 + MY**2 + MZ**2)
    shell = (kmag >= kmin) & (kmag <= kmax)
    amp = np.where(shell, np.power(np.where(shell, kmag, 1.0), alpha), 0.0)
    v = rng.standard_normal((3,) + kmag.shape) + 1j * rng.standard_normal((3,) + kmag.shape)
    phase = np.exp(2j * PI * rng.random(kmag.shape))
    v = v * (amp * phase)[None]
    k2 = KX**2 + KY**2 + KZ**2
    k2s = np.where(k2 > 0, k2, 1.0)
    kdotv = (KX * v[0] + KY * v[1] + KZ * v[2]) / k2s
    v[0] -= kdotv * KX
    v[1] -= kdotv * KY
    v[2] -= kdotv * KZ
    out = np.fft.irfftn(v, s=(nz, ny, nx), axes=(1, 2, 3))
    out -= out.mean(axis=(1, 2, 3), keepdims=True)
    rms = math.sqrt(float(np.mean(np.sum(out**2, axis=0))))
    if rms > 0:
        out /= rms
    return out


def turbulence_ic(n, L=2 * PI, kmin=1, kmax=4, alpha=-1.0, rms_u=0.3, rms_b=0.3, seed=0,
                  rho0=1.0, p0=0.1, B0=(1.0, 0.0, 0.0)):
    """Uniform background plus random-phase divergence-free du, db (u drawn first, then b).

    ``n`` is an int (cube) or an ``(nx, ny, nz)`` triple; returns ``[8, nz, ny, nx]`` float64.
    """
    nx, ny, nz = (n, n, n) if np.isscalar(n) else tuple(n)
    Ls = (L, L, L) if np.isscalar(L) else tuple(L)
    rng = np.random.default_rng(seed)
    du = random_phase_spectrum((nz, ny, nx), Ls, kmin, kmax, alpha, rng) * rms_u
    db = random_phase_spectrum((nz, ny, nx), Ls, kmin, kmax, alpha, rng) * rms_b
    prim = np.empty((8, nz, ny, nx))
    prim[0] = rho0
    prim[1:4] = du
    prim[4] = B0[0] + db[0]
    prim[5] = B0[1] + db[1]
    prim[6] = B0[2] + db[2]
    prim[7] = p0
    return prim


def alfven_wave_ic(n, L=2 * PI, rho0=1.0, p0=0.1, bx0=1.0, db0=0.1, mode=1, cor_angle=0.0):
    """Circularly polarised Alfven wave (``ipert=1`` over ``ifield=3``).

    ``src_compressible/mhdinit.f90:246-251`` (uniform background) and ``:328-342``
    (the wave); an exact nonlinear solution that travels along +x at v_A = bx0/sqrt(rho0).
    """
    nx, ny, nz = (n, n, n) if np.isscalar(n) else tuple(n)
    Lx = L if np.isscalar(L) else L[0]
    x = np.arange(nx) * (Lx / nx)
    kx = 2 * PI / Lx * mode
    s, c = np.sin(kx * x), np.cos(kx * x)
    sa, ca = math.sin(cor_angle), math.cos(cor_angle)
    prim = np.zeros((8, nz, ny, nx))
    prim[0] = rho0
    prim[4] = bx0
    prim[7] = p0
    sr = math.sqrt(rho0)
    prim[6] = prim[6] - db0 * s
    prim[3] = prim[3] + db0 / sr * s
    prim[1] = prim[1] + db0 / sr * c * sa
    prim[4] = prim[4] - db0 * c * sa
    prim[2] = prim[2] + db0 / sr * c * ca
    prim[5] = prim[5] - db0 * c * ca
    return prim


def ensemble_2d(nmembers=64, seed=3, sizes=(128, 256, 512, 1024), kmin=1, kmax=8, rms=0.3):
    """Members of a 2-D compressible Hall-MHD ensemble with uneven grids and parameters.

    For each member, drawn with ``np.random.default_rng(seed)`` in this order: the grid n
    (uniform over ``sizes``), eta and nu (log-uniform on [1e-4, 1e-2]), d_i (uniform on
    [0, 0.1]) and the in-plane field angle theta (uniform on [0, pi/2]).  Returns a list of
    dicts with ``n``, the ``laps_params`` keyword arguments ``kw`` (variant 2-D compressible,
    implicit diffusion, 2/3 mask, cfl 0.4, vardt every 20 steps), ``B0`` and the IC ``seed``;
    ``member_ic(m)`` builds the member's primitive state (random-phase du, db over
    kmin <= |k| <= kmax with rms ``rms``, rho = 1, p = 0.1).
    """
    rng = np.random.default_rng(seed)
    out = []
    for i in range(nmembers):
        n = int(sizes[rng.integers(len(sizes))])
        eta = float(10.0 ** rng.uniform(-4.0, -2.0))
        nu = float(10.0 ** rng.uniform(-4.0, -2.0))
        di = float(rng.uniform(0.0, 0.1))
        th = float(rng.uniform(0.0, PI / 2))
        kw = dict(variant=2, nx=n, ny=n, nz=1, if_resis=1, resistivity=eta, if_visc=1, viscosity=nu,
                  if_Hall=1 if di > 0 else 0, ion_inertial_length=di, dealias_option=1, cfl=0.4,
                  dstep_calcdt=20)
        out.append(dict(n=n, kw=kw, B0=(math.cos(th), math.sin(th), 0.0), seed=1000 * (seed + 1) + i,
                        kmin=kmin, kmax=kmax, rms=rms))
    return out


def member_ic(m):
    """Primitive state ``[8, 1, n, n]`` of one ensemble member from ``ensemble_2d``."""
    n = m["n"]
    return turbulence_ic((n, n, 1), kmin=m["kmin"], kmax=m["kmax"], alpha=-1.0, rms_u=m["rms"], rms_b=m["rms"],
                         seed=m["seed"], B0=m["B0"])


def taylor_green_ic(n, seed=2, kmin=1, kmax=6, alpha=-5.0 / 6.0, rms=1.0, rho0=1.0, p0=1.0):
    """Taylor-Green-like large-scale u and b plus a random-phase component (the 3-D
    incompressible study case).

    u_TG = (sin x cos y cos z, -cos x sin y cos z, 0) and the divergence-free
    b_TG = (cos x sin y sin z, sin x cos y sin z, -2 sin x sin y cos z), each scaled to unit
    rms, plus random-phase divergence-free fields with |k|^alpha amplitudes on
    kmin <= |k| <= kmax (u drawn first, then b, ``np.random.default_rng(seed)``) of unit rms;
    the sums are scaled to rms ``rms``.  rho = rho0, p = p0.  Returns ``[8, n, n, n]``.
    """
    nx, ny, nz = (n, n, n) if np.isscalar(n) else tuple(n)
    x = np.arange(nx) * (2 * PI / nx)
    y = np.arange(ny) * (2 * PI / ny)
    z = np.arange(nz) * (2 * PI / nz)
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    sx, cx_, sy, cy, sz, cz = np.sin(X), np.cos(X), np.sin(Y), np.cos(Y), np.sin(Z), np.cos(Z)
    utg = np.stack([sx * cy * cz, -cx_ * sy * cz, np.zeros_like(X)])
    btg = np.stack([cx_ * sy * sz, sx * cy * sz, -2.0 * sx * sy * cz])

    def unit(v):
        return v / math.sqrt(float(np.mean(np.sum(v ** 2, axis=0))))

    rng = np.random.default_rng(seed)
    du = random_phase_spectrum((nz, ny, nx), (2 * PI,) * 3, kmin, kmax, alpha, rng)
    db = random_phase_spectrum((nz, ny, nx), (2 * PI,) * 3, kmin, kmax, alpha, rng)
    u = unit(unit(utg) + du) * rms
    b = unit(unit(btg) + db) * rms
    prim = np.empty((8, nz, ny, nx))
    prim[0] = rho0
    prim[1:4] = u
    prim[4:7] = b
    prim[7] = p0
    return prim


def ic_phases(ipert: int, nmodex: int, nmodey: int, nmodez: int, seed: int = 0) -> np.ndarray:
    """Phases (radians, uniform on [0, 2 pi)) for the random-phase perturbations of
    ``laps_init_fields``: ipert 6 reads the outward then the inward waves' phases, ipert 7 the
    u, B and rho phases, each in the order of the reference's ``phs`` arrays
    (``src_compressible/mhdinit.f90:523-526,594-597,762-769``).  The reference draws them with
    the Fortran compiler's ``random_number``, whose sequence depends on the compiler; this is a
    seeded ``np.random.default_rng`` stand-in.
    """
    if ipert == 6:
        n = 2 * nmodex * (2 * nmodey + 1) * (2 * nmodez + 1)
    elif ipert == 7:
        n = 3 * (2 * nmodex + 1) * (2 * nmodey + 1) * (2 * nmodez + 1)
    else:
        return np.zeros(0)
    return np.random.default_rng(seed).random(n) * 2 * PI
