"""The GPU engine against closed-form answers, through the C-ABI (no oracle in between).

A Beltrami field B = (sin z, cos z, 0) with u = 0 is force-free (J = B) with a uniform total
pressure, so resistivity is all that acts: each RK stage divides the k = 1 modes by
1 + ts_i eta k^2, ts = (8/15, 2/15, 1/3) dt (rktmod.f90:34-62, implicit branch), and the flow
stays at rest.  The field after ten steps (each step's dt as the engine returns it) must be the
initial one times those factors: FP64 and float-float within 1e-12, the FP32-transform modes
within 1e-6 (their right-hand side is FP32 round-off, not zero)."""
import math

import numpy as np
import pytest

from laps_gb300 import ffi

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec,tol", [(ffi.PREC_FP64, 1e-12), (ffi.PREC_DD, 1e-12), (ffi.PREC_FP32_F64, 1e-6),
                                      (ffi.PREC_FP32, 1e-6)], ids=["fp64", "dd", "fp32_f64", "fp32_dd"])
def test_force_free_field_decays_by_the_implicit_factor(prec, tol):
    n, eta = 16, 0.05
    z = np.arange(n) * (2 * math.pi / n)
    prim = np.zeros((8, n, n, n))
    prim[0] = 1.0
    prim[4] = np.sin(z)[:, None, None]
    prim[5] = np.cos(z)[:, None, None]
    prim[7] = 0.5
    g = ffi.Laps(ffi.params(nx=n, ny=n, nz=n, precision=prec, if_resis=1, resistivity=eta, dealias_option=1, cfl=0.3))
    g.upload_state(prim, primitive=True)
    g.set_time(0.0)
    amp = 1.0
    for _ in range(10):
        t, dt, status = g.step(1)
        assert status == 0
        for ts in (8.0 / 15.0, 2.0 / 15.0, 1.0 / 3.0):
            amp /= 1.0 + ts * dt * eta
    uu, _ = g.download_state()
    g.close()
    assert amp < 0.99
    assert np.abs(uu[4] - amp * prim[4]).max() < tol
    assert np.abs(uu[5] - amp * prim[5]).max() < tol
    assert np.abs(uu[1:4]).max() < tol
