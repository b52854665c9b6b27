"""Ensembles (laps_batch_*): members advanced together by one graph per step.

Every member of a batch must end bitwise equal to the same run advanced alone with
laps_step (the batch replays the very same kernels on the member's own stream), members
keep their own dt / cadence / status (a NaN member stops alone), and a 2-D member matches
the oracle within the 1e-11 bar of the 2-D tests.
"""
import numpy as np
import pytest

from laps_gb300 import ffi
from laps_gb300.ic import ensemble_2d, member_ic, turbulence_ic
from oracle import laps3d

from pairs import rel_l2, state_floor

pytestmark = pytest.mark.gpu


def _members(prec):
    ms = ensemble_2d(nmembers=4, seed=7, sizes=(16, 32, 64))
    out = []
    for m in ms:
        out.append((ffi.params(precision=prec, **m["kw"]), member_ic(m)))
    # a 3-D compressible member in the same batch
    kw3 = dict(if_resis=1, resistivity=5e-4, if_visc=1, viscosity=5e-4, dealias_option=1, cfl=0.4, if_Hall=1,
               ion_inertial_length=0.05, if_AEB=1, radius0=30.0, Ur0=0.3)
    out.append((ffi.params(nx=16, ny=16, nz=16, precision=prec, **kw3), turbulence_ic(16, seed=8, kmax=5)))
    return ms, out


@pytest.mark.parametrize("prec", [ffi.PREC_DD, ffi.PREC_FP32], ids=["dd", "fp32"])
def test_batch_equals_members_alone(prec):
    ms, members = _members(prec)
    b = ffi.Batch([p for p, _ in members])
    for i, (p, prim) in enumerate(members):
        b.members[i].upload_state(prim, primitive=True)
        b.members[i].set_time(0.0)
    t1, d1, s1 = b.step(1)   # the unpruned first steps
    t2, d2, s2 = b.step(24)  # graph replays, crossing the 2-D vardt cadence (every 20 steps)
    assert (s1 == 0).all() and (s2 == 0).all()
    for i, (p, prim) in enumerate(members):
        solo = ffi.Laps(p)
        solo.upload_state(prim, primitive=True)
        solo.set_time(0.0)
        ts, ds, ss = solo.step(25)
        assert ss == 0 and ts == t2[i] and ds == d2[i]
        ub, _ = b.members[i].download_state()
        us, _ = solo.download_state()
        assert np.array_equal(ub, us), i
        solo.close()
    b.close()


def test_batch_member_matches_oracle():
    ms, members = _members(ffi.PREC_DD)
    b = ffi.Batch([p for p, _ in members])
    for i, (p, prim) in enumerate(members):
        b.members[i].upload_state(prim, primitive=True)
        b.members[i].set_time(0.0)
    b.step(25)
    m = ms[1]
    kw = {k: v for k, v in m["kw"].items() if k not in ("variant", "nx", "ny", "nz")}
    o = laps3d.restart2d((m["n"], m["n"]), kw, member_ic(m), 0.0)
    o.dt = 0.0
    for _ in range(25):
        o.step()
    uu, _ = b.members[1].download_state()
    assert rel_l2(uu, o.uu, state_floor(o.uu)).max() < 1e-11
    b.close()


def test_batch_nan_member_stops_alone():
    ms, members = _members(ffi.PREC_DD)
    bad = members[2][1].copy()
    bad[1, 0, 3, 3] = np.nan
    members[2] = (members[2][0], bad)
    b = ffi.Batch([p for p, _ in members])
    for i, (p, prim) in enumerate(members):
        b.members[i].upload_state(prim, primitive=True)
        b.members[i].set_time(0.0)
    t, d, s = b.step(5)
    assert s[2] & ffi.LAPS_STATUS_NAN
    assert all(s[i] == 0 for i in range(len(members)) if i != 2)
    b.close()


def test_batch_errors():
    p = ffi.params(nx=16, ny=16, nz=16)
    q = ffi.params(nx=16, ny=16, nz=16, device=1)
    with pytest.raises(ffi.LapsError):
        ffi.Batch([p, q])  # members on different devices
    b = ffi.Batch([p])
    with pytest.raises(ffi.LapsError):
        b.step(1)  # no state uploaded
    b.close()
