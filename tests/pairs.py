"""Shared helpers: the same seeded case set up in the oracle and on the GPU."""
from __future__ import annotations

import math

import numpy as np

from laps_gb300 import ffi
from laps_gb300.ic import alfven_wave_ic, turbulence_ic
from oracle.laps3d import Laps3DC, Params3D

PI = 3.141592653589793

# the 64^3 plain case: rho=1, p=0.1, B0=(1,0,0), 1<=|k|<=4, |k|^-1, rms 0.3, seed 0,
# gamma 5/3, eta=nu=1e-3 implicit, 2/3 mask, cfl 0.4, no Hall, no expanding box
CONFIG1 = dict(if_resis=1, resistivity=1e-3, if_visc=1, viscosity=1e-3, dealias_option=1, cfl=0.4)
# Hall + expanding box recipe (d_i = 0.05, Ur0/R0 = 0.01, eta = nu = 5e-4)
CONFIG2 = dict(if_resis=1, resistivity=5e-4, if_visc=1, viscosity=5e-4, dealias_option=1, cfl=0.4,
               if_Hall=1, ion_inertial_length=0.05, if_AEB=1, radius0=30.0, Ur0=0.3)


def oracle_params(n, kw) -> Params3D:
    nx, ny, nz = (n, n, n) if np.isscalar(n) else n
    p = Params3D(nx=nx, ny=ny, nz=nz)
    for k, v in kw.items():
        if k in ("precision", "variant"):
            continue
        cur = getattr(p, k)
        setattr(p, k, type(cur)(v) if not isinstance(cur, bool) else bool(v))
    return p


def gpu_params(n, kw, precision=ffi.PREC_FP64):
    nx, ny, nz = (n, n, n) if np.isscalar(n) else n
    return ffi.params(nx=nx, ny=ny, nz=nz, precision=precision, **{k: v for k, v in kw.items() if k != "precision"})


def start_pair(n, kw, prim, precision=ffi.PREC_FP64, t0=0.0):
    """Oracle and GPU started the way the reference restarts: read primitives, evolve_radius(t0),
    conserve, forward transform (mhd.f90:101-122)."""
    o = Laps3DC(oracle_params(n, kw))
    o.initial_calc_conserve_variable(prim)
    o.time = t0
    o.evolve_radius(t0)
    o.transform_uu_real_to_fourier()
    g = ffi.Laps(gpu_params(n, kw, precision))
    g.upload_state(prim, primitive=True)
    g.set_time(t0)
    return o, g


def rel_l2(a, b, floor):
    """Per-field relative L2 error ||a-b|| / max(||b||, floor)."""
    out = []
    for f in range(a.shape[0]):
        nb = float(np.linalg.norm(b[f]))
        out.append(float(np.linalg.norm(a[f] - b[f])) / max(nb, floor))
    return np.array(out)


def state_floor(uu):
    """Norm below which a field counts as zero: errors in it are measured against 1e-3 of
    the state's typical field norm instead of its own (a field that is zero analytically
    holds only round-off)."""
    return 1e-3 * float(np.linalg.norm(uu)) / math.sqrt(uu.shape[0])


def turb(n, **kw):
    return turbulence_ic(n, **kw)


def alfven(n, **kw):
    return alfven_wave_ic(n, **kw)
