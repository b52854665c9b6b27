"""Generate the committed golden fixtures from the oracle (CPU restatement of the reference).

The reference itself cannot run here (Fortran 90 + MPI + FFTW are absent), so these vectors
pin the oracle against regressions and give the GPU tests fixed inputs and outputs; they are
not outputs of the reference binary.  Run:  python tests/golden/make_golden.py
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

from laps_gb300.ic import turbulence_ic  # noqa: E402
from oracle import laps3d  # noqa: E402

CASES = {
    # incompressible 3-D and compressible 2-D cases carry a "variant" key
    "c3di_hall_ebm_16x8x8": ((16, 8, 8), dict(variant=1, if_resis=1, resistivity=5e-4, if_visc=1, viscosity=5e-4,
                                              dealias_option=1, cfl=0.4, if_Hall=1, ion_inertial_length=0.05, if_AEB=1,
                                              radius0=30.0, Ur0=0.3), 4),
    "c2d_zradial_square_32x16": ((32, 16, 1), dict(variant=2, dealias_option=3, cfl=0.4, if_AEB=1, radius0=30.0, Ur0=0.3,
                                                   if_z_radial=1, if_Hall=1, ion_inertial_length=0.05), 25),
    # (nx, ny, nz), parameters, steps
    "c3d_hall_aeb_16x8x8": ((16, 8, 8), dict(if_resis=1, resistivity=5e-4, if_visc=1, viscosity=5e-4, dealias_option=1,
                                             cfl=0.4, if_Hall=1, ion_inertial_length=0.05, if_AEB=1, radius0=30.0,
                                             Ur0=0.3), 4),
    "c3d_filter_explicit_16x8x8": ((16, 8, 8), dict(if_resis=1, resistivity=1e-3, if_resis_exp=1, if_visc=1,
                                                      viscosity=1e-3, if_visc_exp=1, if_conserve_background=1,
                                                      dealias_option=2, cfl=0.3), 4),
    "c3d_corot_16x8x16": ((16, 8, 16), dict(if_resis=1, resistivity=5e-4, if_visc=1, viscosity=5e-4, dealias_option=1,
                                              cfl=0.4, if_Hall=1, ion_inertial_length=0.05, if_AEB=1, radius0=30.0,
                                              Ur0=0.3, if_corotating=1, corotating_angle=0.3), 3),
}


def start(shape, kw, prim):
    """The oracle for the case's variant, started through the restart path."""
    v = kw.get("variant", 0)
    kw = {k: x for k, x in kw.items() if k != "variant"}
    if v == 1:
        return laps3d.restart3di(shape, kw, prim)
    if v == 2:
        return laps3d.restart2d(shape[:2], kw, prim)
    return laps3d.restart(shape, kw, prim)


def run(shape, kw, steps, seed=21):
    prim = turbulence_ic(shape, kmin=1, kmax=3, rms_u=0.3, rms_b=0.3, seed=seed, p0=1.0 if kw.get("variant") == 1 else 0.1)
    o = start(shape, kw, prim)
    dts = []
    for _ in range(steps):
        o.step()
        dts.append(o.dt)
    ave, rms, ru2 = o.calc_rms()
    return dict(prim=prim, uu=o.uu, dts=np.array(dts), time=o.time, ave=ave, rms=rms, rho_u2=ru2,
                divb=o.calc_max_divB(), inv=o.invariants())


def main():
    for name, (shape, kw, steps) in CASES.items():
        out = run(shape, kw, steps)
        np.savez_compressed(HERE / f"{name}.npz", steps=steps, shape=np.array(shape),
                            params=np.array(repr(kw)), **out)
        print(name, out["time"], out["dts"][-1])


if __name__ == "__main__":
    main()
