"""The angle-statistics oracle against the reference's own C tool.

tests/golden/angle_stats_16x8x16.npz holds outputs of theta_ub_zpm_perp_only
(data_process/3D_C/statistics.c:10-356) compiled from the reference tree
(tests/golden/make_angle_stats.py); the restatement in oracle/stats.py must reproduce them.
Where the reference tree is present the tool is also run live on another state.
"""
from pathlib import Path

import numpy as np
import pytest

from oracle import build_ref, stats

GOLDEN = Path(__file__).resolve().parent / "golden" / "angle_stats_16x8x16.npz"
NAMES = ("ub_m1", "ub_m2", "zpm_m1", "zpm_m2")


def test_oracle_matches_reference_fixture():
    d = np.load(GOLDEN)
    for axis in range(3):
        got = stats.angle_statistics(d["prim"], axis)
        for name, g in zip(NAMES, got):
            ref = d[f"{name}_{'xyz'[axis]}"]
            assert ref.shape == g.shape
            assert np.abs(g - ref).max() < 1e-13, (axis, name)
            n = ref.size
            assert np.all(ref[n // 2 + 1:] == 0) and ref[0] == 0
            assert np.all(ref[1 : n // 2 + 1] > 0)


def test_oracle_matches_live_reference():
    if build_ref.build() is None:
        pytest.skip("the reference tree is not available")
    from laps_gb300.ic import turbulence_ic

    prim = turbulence_ic((8, 16, 8), seed=23, kmax=3, rms_u=0.2, rms_b=0.6)
    prim[4] += 0.7
    prim[6] -= 0.2
    for axis in range(3):
        ref = build_ref.run_angle_statistics(prim, axis)
        got = stats.angle_statistics(prim, axis)
        for r, g in zip(ref, got):
            assert np.abs(g - r).max() < 1e-13
