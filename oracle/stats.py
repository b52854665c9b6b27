"""CPU restatement of the reference's angle statistics (test infrastructure).

The oracle of ``laps_angle_statistics``: the perpendicular angles between the increments
of u and b = B / sqrt(<rho>), and of z+ = u - b and z- = u + b, at lags 1 .. n/2 along one
axis, following theta_ub_zpm_perp_only (data_process/3D_C/statistics.c:10-356) with numpy
arrays in place of its point loop: means (:86-101), increments with periodic wrap
(:149-171), parts perpendicular to b0 (mathlib.c:47-60, statistics.c:172-181), method 1 and
method 2 (:183-198, :338-349).  Input: primitive fields ``[8, nz, ny, nx]``.
"""
from __future__ import annotations

import numpy as np


def _perp(v, b0):
    d = v[0] * b0[0] + v[1] * b0[1] + v[2] * b0[2]
    return np.stack([v[0] - b0[0] * d, v[1] - b0[1] * d, v[2] - b0[2] * d])


def _pair(a, b, b0):
    ap, bp = _perp(a, b0), _perp(b, b0)
    an = np.sqrt(ap[0] ** 2 + ap[1] ** 2 + ap[2] ** 2)
    bn = np.sqrt(bp[0] ** 2 + bp[1] ** 2 + bp[2] ** 2)
    c = np.stack([ap[1] * bp[2] - ap[2] * bp[1], ap[2] * bp[0] - ap[0] * bp[2], ap[0] * bp[1] - ap[1] * bp[0]])
    cn = np.sqrt(c[0] ** 2 + c[1] ** 2 + c[2] ** 2)
    ok = (an > 0) & (bn > 0)
    with np.errstate(invalid="ignore", divide="ignore"):
        m1 = np.arcsin(cn[ok] / (an[ok] * bn[ok])).sum() / ok.sum()
        m2 = np.arcsin(cn.sum() / (an * bn).sum())
    return m1, m2


def angle_statistics(prim: np.ndarray, axis: int):
    """[ub method 1, ub method 2, zpm method 1, zpm method 2], n_axis values each."""
    rho0 = prim[0].mean()
    B0 = np.array([prim[4].mean(), prim[5].mean(), prim[6].mean()])
    b0 = B0 / np.sqrt((B0**2).sum())
    ax = 2 - axis  # numpy axis of x, y, z in [nz, ny, nx]
    n = prim.shape[1 + ax]
    out = [np.zeros(n) for _ in range(4)]
    u, B = prim[1:4], prim[4:7]
    for l in range(1, n // 2 + 1):
        du = np.roll(u, -l, axis=1 + ax) - u
        db = (np.roll(B, -l, axis=1 + ax) - B) / np.sqrt(rho0)
        out[0][l], out[1][l] = _pair(du, db, b0)
        out[2][l], out[3][l] = _pair(du - db, du + db, b0)
    return out
