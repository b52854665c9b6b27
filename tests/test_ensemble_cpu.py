"""The 2-D ensemble recipe (64 members, seed 3): reproducible, with every drawn value in its
stated range, and members' initial states with the drawn mean field."""
import numpy as np

from laps_gb300.ic import ensemble_2d, member_ic


def test_ensemble_recipe():
    a, b = ensemble_2d(), ensemble_2d()
    assert a == b and len(a) == 64
    for m in a:
        kw = m["kw"]
        assert m["n"] in (128, 256, 512, 1024) and kw["nx"] == kw["ny"] == m["n"] and kw["nz"] == 1
        assert 1e-4 <= kw["resistivity"] <= 1e-2 and 1e-4 <= kw["viscosity"] <= 1e-2
        assert 0.0 <= kw["ion_inertial_length"] <= 0.1
        th = np.arctan2(m["B0"][1], m["B0"][0])
        assert 0.0 <= th <= np.pi / 2
    small = ensemble_2d(nmembers=3, seed=5, sizes=(16,))
    p = member_ic(small[0])
    assert p.shape == (8, 1, 16, 16)
    assert np.allclose([p[4].mean(), p[5].mean(), p[6].mean()], small[0]["B0"], atol=1e-12)
    u2 = np.mean(p[1] ** 2 + p[2] ** 2 + p[3] ** 2)
    assert abs(np.sqrt(u2) - 0.3) < 1e-12
