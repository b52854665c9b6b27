"""The C++/OpenMP restatement (oracle O2, the benchmark's CPU baseline) against the numpy
restatement: the Hall + expanding-box case and the plain case agree after several steps
within 1e-12 relative L2 per field, dt and time within 1e-13."""
import numpy as np
import pytest

from laps_gb300.ic import turbulence_ic
from oracle import laps3d, laps3d_omp

from pairs import CONFIG1, CONFIG2, rel_l2, state_floor


@pytest.mark.parametrize("case,shape", [("config2", 32), ("config1", (32, 16, 8)), ("config2", (16, 32, 64))])
def test_o2_matches_numpy_oracle(case, shape):
    kw = {"config1": CONFIG1, "config2": CONFIG2}[case]
    prim = turbulence_ic(shape, seed=21, kmax=3, rms_u=0.4, rms_b=0.4)
    o = laps3d.restart(shape, kw, prim)
    o.dt = 0.0
    r = laps3d_omp.Run(shape, kw)
    r.set_state(prim)
    for _ in range(3):
        o.step()
    t, dt = r.step(3)
    assert abs(dt - o.dt) <= 1e-13 * o.dt and abs(t - o.time) <= 1e-13 * o.time
    uu = r.state()
    err = rel_l2(uu, o.uu, state_floor(o.uu))
    assert err.max() < 1e-12, err
    r.close()


def test_o2_rejects_options_it_does_not_cover():
    with pytest.raises(ValueError):
        laps3d_omp.Run(16, dict(CONFIG2, if_corotating=1))
