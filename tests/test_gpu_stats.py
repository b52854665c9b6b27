"""laps_angle_statistics on the device against the reference tool's outputs and the oracle.

The golden fixture holds what the reference's own theta_ub_zpm_perp_only
(data_process/3D_C/statistics.c:10-356) computed for a seeded state; the device, given the
same state, must return the same four arrays per axis.  A larger state checks the device
against the oracle restatement (oracle/stats.py) in every arithmetic mode.
"""
from pathlib import Path

import numpy as np
import pytest

from laps_gb300 import ffi
from laps_gb300.ic import turbulence_ic
from oracle import stats

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden" / "angle_stats_16x8x16.npz"
NAMES = ("ub_m1", "ub_m2", "zpm_m1", "zpm_m2")


@pytest.mark.parametrize("prec", [ffi.PREC_FP64, ffi.PREC_DD, ffi.PREC_FP32], ids=["fp64", "dd", "fp32"])
def test_angle_statistics_match_reference_tool(prec):
    d = np.load(GOLDEN)
    prim = d["prim"]
    nz, ny, nx = prim.shape[1:]
    g = ffi.Laps(ffi.params(nx=nx, ny=ny, nz=nz, precision=prec))
    g.upload_state(prim, primitive=True)
    for axis in range(3):
        got = g.angle_statistics(axis)
        for k, name in enumerate(NAMES):
            ref = d[f"{name}_{'xyz'[axis]}"]
            assert np.abs(got[k] - ref).max() < 1e-12, (axis, name)


@pytest.mark.parametrize("variant", [ffi.VARIANT_3DC, ffi.VARIANT_3DI], ids=["3dc", "3di"])
def test_angle_statistics_match_oracle_64(variant):
    prim = turbulence_ic((64, 32, 64), seed=29, kmax=6, rms_u=0.3, rms_b=0.4)
    prim[4] += 0.5
    prim[5] -= 0.5
    g = ffi.Laps(ffi.params(nx=64, ny=32, nz=64, variant=variant, precision=ffi.PREC_FP64))
    g.upload_state(prim, primitive=True)
    for axis in range(3):
        got = g.angle_statistics(axis)
        ref = stats.angle_statistics(prim, axis)
        for k in range(4):
            assert np.abs(got[k] - ref[k]).max() < 1e-12, (axis, k)


def test_angle_statistics_rejects_bad_axis():
    g = ffi.Laps(ffi.params(nx=16, ny=8, nz=8))
    with pytest.raises(ffi.LapsError):
        g._ck(g.lib.laps_angle_statistics(g.h, 3, None))
