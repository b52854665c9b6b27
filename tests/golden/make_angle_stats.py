"""Generate the golden fixture of the angle statistics from the reference's own C tool.

theta_ub_zpm_perp_only (data_process/3D_C/statistics.c:10-356) is compiled from the reference
tree by oracle/build_ref.py and run on a seeded primitive state for each axis; the fixture
holds the state and the four arrays per axis the tool wrote (the contents of its
theta_{ub,zpm}_perp_only_l{x,y,z}_method{1,2}_000.dat files).  Run in a tree that has the
reference:  python tests/golden/make_angle_stats.py
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

from laps_gb300.ic import turbulence_ic  # noqa: E402
from oracle import build_ref  # noqa: E402

SHAPE = (16, 8, 16)  # nx, ny, nz (powers of two: the engine's grids)


def make():
    prim = turbulence_ic(SHAPE, seed=17, kmax=4, rms_u=0.4, rms_b=0.5)
    prim[5] += 0.4  # <B> off the x axis
    out = {"prim": prim}
    for axis in range(3):
        res = build_ref.run_angle_statistics(prim, axis)
        for name, arr in zip(("ub_m1", "ub_m2", "zpm_m1", "zpm_m2"), res):
            out[f"{name}_{'xyz'[axis]}"] = arr
    np.savez_compressed(HERE / "angle_stats_16x8x16.npz", **out)


if __name__ == "__main__":
    make()
